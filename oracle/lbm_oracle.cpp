// lbm_oracle.cpp — TEST INFRASTRUCTURE ONLY (the oracle).
//
// CPU restatement of taktoa/chemsim's D2Q9 lattice-Boltzmann step
// (src/lbm.rs), used by the test-suite, __graft_entry__.smoke() and the CPU
// legs of bench.py as the checker.  Nothing in the shipped library links,
// loads or calls this file.
//
// PARITY UNPINNED: the reference cannot run on this machine (it is Rust over
// ArrayFire 3.6, and neither a Rust toolchain nor ArrayFire is installed), and
// it ships no tests, golden vectors or fixtures.  This restatement is instead
// cross-checked bit-for-bit against a second, independent restatement written
// in numpy (tests/golden/make_golden.py), which executes lbm.rs's ArrayFire
// call sequence literally (scipy's convolve2d standing in for af::convolve2,
// np.where for af::replace), and against physics known-answer tests.
//
// What follows which reference line:
//   D2Q9 weights / velocities / direction order ... src/lbm.rs:202-282
//   opposite-direction swap ....................... src/lbm.rs:298-309
//   isothermal speed of sound cs = dx/(sqrt(3) dt)  src/lbm.rs:83-85
//   compute_equilibrium (op order kept) ........... src/lbm.rs:43-71
//   density / momentum_density / velocity ......... src/lbm.rs:117-149
//   BGK f* = f + (f - feq) * (-dt/tau) ............ src/lbm.rs:350-364
//   TRT (incl. swap_equilibrium's use of f) ....... src/lbm.rs:399-446, 311-322
//   stream = convolve2(f_i, stencil_i^T) .......... src/lbm.rs:716-729
//   bounce_back = replace(swap(f), geometry, f) ... src/lbm.rs:741-751
//   step = stream -> bounce_back -> collide ....... src/lbm.rs:694-714
//   is_unstable = min f_eq[0] < 0 ................. src/lbm.rs:815-818
//
// Every floating-point operation is written in the order lbm.rs evaluates it,
// one rounding per operation; the file must be compiled with
// -ffp-contract=off (and without -ffast-math) so no FMA is formed.
//
// Extensions with no reference counterpart (periodic / half-way wall axes,
// half-way solid bounce-back, the XY frame, Guo body forcing) follow the
// definitions in include/lbm_cuda.h.

#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/lbm_cuda.h"

namespace {

// src/lbm.rs:216-238 — velocity set in direction order 0..8.
const int CX[9] = {0, 1, 0, -1, 0, 1, -1, -1, 1};
const int CY[9] = {0, 0, 1, 0, -1, 1, 1, -1, -1};
// src/lbm.rs:298-309 — swap_populations: 1<->3, 2<->4, 5<->7, 6<->8.
const int OPP[9] = {0, 3, 4, 1, 2, 7, 8, 5, 6};

// src/lbm.rs:240-280 — the 3x3 streaming stencils, row-major as written.
const int STENCIL[9][9] = {
    {0, 0, 0, 0, 1, 0, 0, 0, 0}, {0, 0, 0, 1, 0, 0, 0, 0, 0},
    {0, 0, 0, 0, 0, 0, 0, 1, 0}, {0, 0, 0, 0, 0, 1, 0, 0, 0},
    {0, 1, 0, 0, 0, 0, 0, 0, 0}, {0, 0, 0, 0, 0, 0, 1, 0, 0},
    {0, 0, 0, 0, 0, 0, 0, 0, 1}, {0, 0, 1, 0, 0, 0, 0, 0, 0},
    {1, 0, 0, 0, 0, 0, 0, 0, 0},
};

// Grid displacement (dcol, drow) of direction i.
//  REF frame: convolve2(f_i, S_i^T) with ArrayFire's true (flipped-kernel)
//  convolution moves plane i by (drow, dcol) = (-cx, +cy) (src/lbm.rs:233-269
//  with src/matrix.rs:24-30: row = y, column = x).
//  XY frame: (dcol, drow) = (+cx, +cy).
inline void displacement(int frame_xy, int i, int& dcol, int& drow) {
    if (frame_xy) { dcol = CX[i]; drow = CY[i]; }
    else          { dcol = CY[i]; drow = -CX[i]; }
}

template <class T>
struct Params {
    int w = 0, h = 0, flags = 0, collision = LBM_COLLISION_BGK;
    T wt[9];
    T k1, k2, k3;         // 1/cs2, 1/(2 cs4), -1/(2 cs2)   (src/lbm.rs:54-66)
    T cs2;
    T bgk_factor;         // -dt/tau                          (src/lbm.rs:357)
    T omega_p, omega_m;   // 1/tau_plus, 1/tau_minus          (src/lbm.rs:430-431)
    T trt_scale;          // -dt * 0.5                        (src/lbm.rs:441)
    bool force = false;
    T fx, fy, hfx, hfy;   // F and F/2
    T guo;                // 1 - 1/(2 tau)
    T inv_cs4;
};

template <class T>
Params<T> make_params(int w, int h, int flags, int collision, double tau,
                      double tau_minus, double dx, double dt, double fx,
                      double fy) {
    Params<T> P;
    P.w = w; P.h = h; P.flags = flags; P.collision = collision;
    // src/lbm.rs:205-215: weights written as 16.0/36.0 etc. in Scalar.
    const T n[9] = {T(16), T(4), T(4), T(4), T(4), T(1), T(1), T(1), T(1)};
    for (int i = 0; i < 9; ++i) P.wt[i] = n[i] / T(36);
    const T tdx = T(dx), tdt = T(dt);
    // src/lbm.rs:83-85: cs = dx / (sqrt(3) * dt), all in Scalar.
    const T cs = tdx / (std::sqrt(T(3)) * tdt);
    const T cs2 = cs * cs;
    const T cs4 = cs2 * cs2;
    P.cs2 = cs2;
    P.k1 = T(1) / cs2;
    P.k2 = T(1) / (T(2) * cs4);
    P.k3 = T(-1) / (T(2) * cs2);
    const T ttau = T(tau);
    P.bgk_factor = -tdt / ttau;
    P.omega_p = T(1) / ttau;
    P.omega_m = T(1) / T(tau_minus);
    P.trt_scale = -tdt * T(0.5);
    P.fx = T(fx); P.fy = T(fy);
    P.force = (fx != 0.0 || fy != 0.0);
    P.hfx = P.fx * T(0.5); P.hfy = P.fy * T(0.5);
    P.guo = T(1) - T(1) / (T(2) * ttau);
    P.inv_cs4 = T(1) / cs4;
    return P;
}

// src/lbm.rs:117-121 (density) and :123-131 (momentum_density), op order kept.
template <class T>
inline void moments_ref(const T f[9], T& rho, T& mx, T& my) {
    rho = T(0);
    for (int i = 0; i < 9; ++i) rho = rho + f[i];
    mx = T(0);
    my = T(0);
    for (int i = 0; i < 9; ++i) {
        mx = mx + f[i] * T(CX[i]);
        my = my + f[i] * T(CY[i]);
    }
}

// src/lbm.rs:43-71 for one cell and one direction.
template <class T>
inline T equilibrium_ref(const Params<T>& P, int i, T rho, T vx, T vy, T v2) {
    const T vc = vx * T(CX[i]) + vy * T(CY[i]);
    const T vc2 = vc * vc;
    const T sum = ((T(1) + vc * P.k1) + vc2 * P.k2) + v2 * P.k3;
    return (rho * P.wt[i]) * sum;
}

// Guo source term for direction i (no reference counterpart).
template <class T>
inline T guo_source(const Params<T>& P, int i, T vx, T vy) {
    const T cx = T(CX[i]), cy = T(CY[i]);
    const T vc = vx * cx + vy * cy;
    const T a = ((cx - vx) * P.fx + (cy - vy) * P.fy) * P.k1;
    const T b = (vc * (cx * P.fx + cy * P.fy)) * P.inv_cs4;
    return (P.guo * P.wt[i]) * (a + b);
}

// Collision of one cell: Lattice::equilibrium (src/lbm.rs:156-160) then
// BGK::evaluate (src/lbm.rs:350-364) or TRT::evaluate (src/lbm.rs:399-446).
template <class T>
inline void collide_cell(const Params<T>& P, const T f[9], T out[9]) {
    T rho, mx, my;
    moments_ref(f, rho, mx, my);
    if (P.force) { mx = mx + P.hfx; my = my + P.hfy; }
    const T inv = T(1) / rho;                 // Matrix::recip, src/matrix.rs:133-136
    const T vx = inv * mx;
    const T vy = inv * my;
    const T v2 = vx * vx + vy * vy;
    T feq[9];
    for (int i = 0; i < 9; ++i) feq[i] = equilibrium_ref(P, i, rho, vx, vy, v2);
    if (P.collision == LBM_COLLISION_TRT) {
        for (int i = 0; i < 9; ++i) {
            const int o = OPP[i];
            // swap_populations: f_sw[i] = f[opp(i)]; swap_equilibrium keeps
            // f_eq[0] but fills entries 1..8 from the populations f[opp(i)]
            // (src/lbm.rs:311-322) — reproduced as written.
            const T f_sw = f[o];
            const T feq_sw = (i == 0) ? feq[0] : f[o];
            const T f_p = f[i] + f_sw;
            const T f_m = f[i] - f_sw;
            const T feq_p = feq[i] + feq_sw;
            const T feq_m = feq[i] - feq_sw;
            const T omega = ((f_p - feq_p) * P.omega_p + (f_m - feq_m) * P.omega_m) * P.trt_scale;
            out[i] = f[i] + omega;
        }
    } else {
        for (int i = 0; i < 9; ++i) out[i] = f[i] + (f[i] - feq[i]) * P.bgk_factor;
    }
    if (P.force) {
        for (int i = 0; i < 9; ++i) out[i] = out[i] + guo_source(P, i, vx, vy);
    }
}

enum SourceKind { SRC_CELL = 0, SRC_ZERO = 1, SRC_BOUNCE = 2 };

// Classifies the pull source of direction i at (x, y) and returns its index.
template <class T>
inline SourceKind pull_source(const Params<T>& P, const uint8_t* solid, int i,
                              int x, int y, int64_t& idx) {
    int dcol, drow;
    displacement(P.flags & LBM_FRAME_XY, i, dcol, drow);
    int sx = x - dcol, sy = y - drow;
    bool zero = false, bounce = false;
    const int xm = P.flags & 0x3, ym = (P.flags >> 2) & 0x3;
    if (sx < 0 || sx >= P.w) {
        if (xm == LBM_X_PERIODIC) sx = (sx + P.w) % P.w;
        else if (xm == LBM_X_WALL) bounce = true;
        else zero = true;
    }
    if (sy < 0 || sy >= P.h) {
        if (ym == 1) sy = (sy + P.h) % P.h;
        else if (ym == 2) bounce = true;
        else zero = true;
    }
    if (bounce) return SRC_BOUNCE;
    if (zero) return SRC_ZERO;
    idx = int64_t(sy) * P.w + sx;
    if (solid && (P.flags & LBM_SOLID_HALFWAY) && solid[idx]) return SRC_BOUNCE;
    return SRC_CELL;
}

// One fused step over all cells (the per-cell form of src/lbm.rs:694-714).
template <class T>
void step_fused(const Params<T>& P, const uint8_t* solid, const T* src, T* dst,
                int threads) {
    const int64_t n = int64_t(P.w) * P.h;
    const bool halfway = (P.flags & LBM_SOLID_HALFWAY) != 0;
#pragma omp parallel for schedule(static) num_threads(threads)
    for (int y = 0; y < P.h; ++y) {
        for (int x = 0; x < P.w; ++x) {
            const int64_t c = int64_t(y) * P.w + x;
            if (solid && halfway && solid[c]) {
                for (int i = 0; i < 9; ++i) dst[i * n + c] = src[i * n + c];
                continue;
            }
            T f[9];
            for (int i = 0; i < 9; ++i) {
                int64_t s = 0;
                switch (pull_source(P, solid, i, x, y, s)) {
                    case SRC_CELL: f[i] = src[i * n + s]; break;
                    case SRC_ZERO: f[i] = T(0); break;
                    default: f[i] = src[OPP[i] * n + c]; break;
                }
            }
            if (solid && !halfway && solid[c]) {
                // bounce_back: solid nodes take the swapped populations.
                T g[9];
                for (int i = 0; i < 9; ++i) g[i] = f[OPP[i]];
                for (int i = 0; i < 9; ++i) f[i] = g[i];
            }
            T out[9];
            collide_cell(P, f, out);
            for (int i = 0; i < 9; ++i) dst[i * n + c] = out[i];
        }
    }
}

// The same step executed the way lbm.rs drives ArrayFire: full-plane passes
// that materialise after each convolve2 and each replace, and a collide pass
// per output direction that re-derives rho and u from all nine planes (the
// lazily evaluated JIT tree of src/lbm.rs:731-739).  Produces the same bits as
// step_fused; it exists as the reference-structured CPU baseline.
template <class T>
void step_structured(const Params<T>& P, const uint8_t* solid, T* f, T* tmp,
                     int threads) {
    const int64_t n = int64_t(P.w) * P.h;
    const bool literal_conv =
        (P.flags & (0xF | LBM_FRAME_XY | LBM_SOLID_HALFWAY)) == 0;
    const bool halfway = (P.flags & LBM_SOLID_HALFWAY) != 0;
    // stream: one pass per plane (src/lbm.rs:716-729).
    for (int i = 0; i < 9; ++i) {
        const T* in = f + i * n;
        T* out = tmp + i * n;
        if (literal_conv) {
            // af::convolve2(f_i, S_i^T): out[r][c] = sum_{m,n} in[r-m+1][c-n+1] * K[m][n],
            // zero outside, with K = S_i^T built from the stencil exactly as
            // lbm.rs writes it (Matrix::new reads the 9 values row-major).
            T K[3][3];
            for (int m = 0; m < 3; ++m)
                for (int q = 0; q < 3; ++q) K[m][q] = T(STENCIL[i][q * 3 + m]);
#pragma omp parallel for schedule(static) num_threads(threads)
            for (int r = 0; r < P.h; ++r) {
                for (int c = 0; c < P.w; ++c) {
                    T acc = T(0);
                    for (int m = 0; m < 3; ++m) {
                        const int rr = r - m + 1;
                        for (int q = 0; q < 3; ++q) {
                            const int cc = c - q + 1;
                            const T v = (rr >= 0 && rr < P.h && cc >= 0 && cc < P.w)
                                            ? in[int64_t(rr) * P.w + cc] : T(0);
                            acc = acc + v * K[m][q];
                        }
                    }
                    out[int64_t(r) * P.w + c] = acc;
                }
            }
        } else {
#pragma omp parallel for schedule(static) num_threads(threads)
            for (int y = 0; y < P.h; ++y) {
                for (int x = 0; x < P.w; ++x) {
                    const int64_t c = int64_t(y) * P.w + x;
                    if (solid && halfway && solid[c]) { out[c] = in[c]; continue; }
                    int64_t s = 0;
                    switch (pull_source(P, solid, i, x, y, s)) {
                        case SRC_CELL: out[c] = in[s]; break;
                        case SRC_ZERO: out[c] = T(0); break;
                        default: out[c] = f[OPP[i] * n + c]; break;
                    }
                }
            }
        }
    }
    // bounce_back: replace(swap(f), geometry, f), one pass per plane
    // (src/lbm.rs:741-751).
    if (solid && !halfway) {
        for (int i = 0; i < 9; ++i) {
            T* out = f + i * n;
            const T* sw = tmp + OPP[i] * n;
            const T* orig = tmp + i * n;
#pragma omp parallel for schedule(static) num_threads(threads)
            for (int64_t c = 0; c < n; ++c) out[c] = solid[c] ? sw[c] : orig[c];
        }
        std::memcpy(tmp, f, sizeof(T) * 9 * n);
    }
    // collide: each output plane evaluates its own expression tree over all
    // nine input planes (src/lbm.rs:731-739 -> :156-160 -> :350-364).
    for (int i = 0; i < 9; ++i) {
        T* out = f + i * n;
#pragma omp parallel for schedule(static) num_threads(threads)
        for (int64_t c = 0; c < n; ++c) {
            T g[9], o[9];
            for (int k = 0; k < 9; ++k) g[k] = tmp[k * n + c];
            if (solid && halfway && solid[c]) { out[c] = g[i]; continue; }
            collide_cell(P, g, o);
            out[c] = o[i];
        }
    }
}

template <class T>
void moments_state(const Params<T>& P, const T* f, T* rho, T* ux, T* uy) {
    const int64_t n = int64_t(P.w) * P.h;
    for (int64_t c = 0; c < n; ++c) {
        T g[9];
        for (int i = 0; i < 9; ++i) g[i] = f[i * n + c];
        T r, mx, my;
        moments_ref(g, r, mx, my);
        if (P.force) { mx = mx - P.hfx; my = my - P.hfy; }
        const T inv = T(1) / r;
        rho[c] = r;
        ux[c] = inv * mx;
        uy[c] = inv * my;
    }
}

template <class T>
void equilibrium_fields(const Params<T>& P, const T* rho, const T* ux,
                        const T* uy, T* f) {
    const int64_t n = int64_t(P.w) * P.h;
    for (int64_t c = 0; c < n; ++c) {
        const T v2 = ux[c] * ux[c] + uy[c] * uy[c];   // src/lbm.rs:53
        for (int i = 0; i < 9; ++i)
            f[i * n + c] = equilibrium_ref(P, i, rho[c], ux[c], uy[c], v2);
    }
}

template <class T>
void health_state(const Params<T>& P, const T* f, double* out6, int64_t* nonfinite) {
    const int64_t n = int64_t(P.w) * P.h;
    double mass = 0, px = 0, py = 0;
    double minf = std::numeric_limits<double>::infinity();
    double mineq = std::numeric_limits<double>::infinity();
    int64_t bad = 0;
    for (int64_t c = 0; c < n; ++c) {
        T g[9];
        for (int i = 0; i < 9; ++i) {
            g[i] = f[i * n + c];
            if (!std::isfinite(double(g[i]))) ++bad;
            else if (double(g[i]) < minf) minf = double(g[i]);
        }
        T r, mx, my;
        moments_ref(g, r, mx, my);
        mass += double(r); px += double(mx); py += double(my);
        const T inv = T(1) / r;
        const T vx = inv * mx, vy = inv * my;
        const T v2 = vx * vx + vy * vy;
        const double e0 = double(equilibrium_ref(P, 0, r, vx, vy, v2));
        if (e0 < mineq || std::isnan(e0)) mineq = std::isnan(e0) ? mineq : e0;
    }
    out6[0] = mass; out6[1] = px; out6[2] = py; out6[3] = minf; out6[4] = mineq;
    *nonfinite = bad;
}

template <class T>
int run_steps(int w, int h, int flags, int collision, double tau,
              double tau_minus, double dx, double dt, double fx, double fy,
              const uint8_t* solid, void* fv, int nsteps, int structured,
              int threads) {
    if (w <= 0 || h <= 0 || nsteps < 0) return LBM_ERR_INVALID_ARGUMENT;
    const Params<T> P = make_params<T>(w, h, flags, collision, tau, tau_minus,
                                       dx, dt, fx, fy);
    T* f = static_cast<T*>(fv);
    const size_t count = size_t(9) * w * h;
    std::vector<T> tmp(count);
    for (int s = 0; s < nsteps; ++s) {
        if (structured) {
            step_structured(P, solid, f, tmp.data(), threads);
        } else {
            step_fused(P, solid, f, tmp.data(), threads);
            std::memcpy(f, tmp.data(), sizeof(T) * count);
        }
    }
    return LBM_OK;
}

}  // namespace

extern "C" {

// Advance nsteps on a host SoA population array (9*w*h, f32 when prec ==
// LBM_F32, f64 when prec == LBM_F64), in place.
int orc_step(int prec, int w, int h, int flags, int collision, double tau,
             double tau_minus, double dx, double dt, double fx, double fy,
             const uint8_t* solid, void* f, int nsteps, int structured,
             int threads) {
    if (threads <= 0) threads = 1;
    if (prec == LBM_F32)
        return run_steps<float>(w, h, flags, collision, tau, tau_minus, dx, dt,
                                fx, fy, solid, f, nsteps, structured, threads);
    if (prec == LBM_F64)
        return run_steps<double>(w, h, flags, collision, tau, tau_minus, dx, dt,
                                 fx, fy, solid, f, nsteps, structured, threads);
    return LBM_ERR_INVALID_ARGUMENT;
}

// compute_equilibrium over whole fields (src/lbm.rs:43-71).
int orc_equilibrium(int prec, int w, int h, double dx, double dt,
                    const void* rho, const void* ux, const void* uy, void* f) {
    if (prec == LBM_F32) {
        auto P = make_params<float>(w, h, 0, 0, 1.0, 1.0, dx, dt, 0, 0);
        equilibrium_fields(P, (const float*)rho, (const float*)ux, (const float*)uy, (float*)f);
        return LBM_OK;
    }
    if (prec == LBM_F64) {
        auto P = make_params<double>(w, h, 0, 0, 1.0, 1.0, dx, dt, 0, 0);
        equilibrium_fields(P, (const double*)rho, (const double*)ux, (const double*)uy, (double*)f);
        return LBM_OK;
    }
    return LBM_ERR_INVALID_ARGUMENT;
}

// density and velocity of a state (src/lbm.rs:117-149); u = (j - F/2)/rho
// when a force is given.
int orc_moments(int prec, int w, int h, double fx, double fy, const void* f,
                void* rho, void* ux, void* uy) {
    if (prec == LBM_F32) {
        auto P = make_params<float>(w, h, 0, 0, 1.0, 1.0, 1.0, 1.0, fx, fy);
        moments_state(P, (const float*)f, (float*)rho, (float*)ux, (float*)uy);
        return LBM_OK;
    }
    if (prec == LBM_F64) {
        auto P = make_params<double>(w, h, 0, 0, 1.0, 1.0, 1.0, 1.0, fx, fy);
        moments_state(P, (const double*)f, (double*)rho, (double*)ux, (double*)uy);
        return LBM_OK;
    }
    return LBM_ERR_INVALID_ARGUMENT;
}

// Health reduction: out6 = {mass, momentum_x, momentum_y, min f, min f_eq[0], 0}.
int orc_health(int prec, int w, int h, double dx, double dt, const void* f,
               double* out6, int64_t* nonfinite) {
    if (prec == LBM_F32) {
        auto P = make_params<float>(w, h, 0, 0, 1.0, 1.0, dx, dt, 0, 0);
        health_state(P, (const float*)f, out6, nonfinite);
        return LBM_OK;
    }
    if (prec == LBM_F64) {
        auto P = make_params<double>(w, h, 0, 0, 1.0, 1.0, dx, dt, 0, 0);
        health_state(P, (const double*)f, out6, nonfinite);
        return LBM_OK;
    }
    return LBM_ERR_INVALID_ARGUMENT;
}

int orc_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

}  // extern "C"
