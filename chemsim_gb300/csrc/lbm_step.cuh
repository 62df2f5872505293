// lbm_step.cuh — the fused D2Q9 step kernel (sm_103a).
//
// One launch = one time step of State::step (taktoa/chemsim
// src/lbm.rs:694-714): pull streaming (stream, :716-729), bounce-back
// (:741-751, or its half-way variant), moments, equilibrium
// (compute_equilibrium, :43-71) and relaxation (BGK :350-364 / TRT
// :399-446), fused so each population is read once and written once.
//
// Layout: 9 structure-of-arrays planes, rows of `pitch` elements (a multiple
// of 128 bytes), x contiguous.  A warp owns 32*V consecutive cells of one row;
// each lane loads V cells of a plane with one aligned vector load (16 bytes
// for f32 V=4, f64 V=2, 16-bit V=8).  The +-1 column shifts of the pull are
// realigned in registers with warp shuffles (16-bit values stay packed two
// per register and shift by byte permutes), so every global load is an
// aligned, coalesced vector; only the two lanes at a warp's ends fetch one
// extra scalar (an L1/L2 hit).  Row shifts are plain row offsets.
//
// Each step is one launch.  Per (row, warp tile) flag: 0 = the interior path
// (the 3 x (32V + 2) neighbourhood is fluid and inside the lattice, or wraps
// at periodic edges: no boundary logic), 2 = the same for the partial last
// tile of a periodic row, 1 = the general path with the full boundary
// treatment (non-periodic edges), 3 = solids nearby, every source cell inside
// the lattice.  Tiles 1 are listed and run first (the general path); tiles 3
// run in place on the interior code with per-lane link masks where the
// lattice has them (f32, 16-bit at 8 cells per thread), else they are listed
// too and take the general path without edge handling.  Interior warps also
// prefetch into L2 the rows that warps
// further down the row-major wavefront will pull.  The flags and the list
// are rebuilt whenever the geometry or the tile width changes.
#pragma once

#include <array>
#include <type_traits>

#include "lbm_common.cuh"
#include "lbm_pair.cuh"

namespace lbmk {

constexpr unsigned kFull = 0xffffffffu;

// 16-bit storage keeps values packed two per register through the shifts
// (LBM_PACKED16 = 0 selects the plain form).  At 8 cells per thread the
// periodic-edge path collides its pairs in a loop that is not unrolled
// (LBM_ROLL_WRAP; the general paths always do): less code for the instruction
// cache, measured 1% faster; unrolled is faster for the interior path.
#ifndef LBM_PACKED16
#define LBM_PACKED16 1
#endif
#ifndef LBM_ROLL_INTERIOR
#define LBM_ROLL_INTERIOR 0
#endif
#ifndef LBM_ROLL_WRAP
#define LBM_ROLL_WRAP 1
#endif

template <class S, int V>
struct VecIO {
    static constexpr int BYTES = int(sizeof(S)) * V;
    static_assert(BYTES == 4 || BYTES == 8 || BYTES == 16 || BYTES == 32, "vector width");
    __device__ __forceinline__ static void load(const S* p, S (&out)[V]) {
        if constexpr (BYTES == 32) {
            const uint4* q = reinterpret_cast<const uint4*>(p);
            uint4 r[2] = {__ldg(q), __ldg(q + 1)};
            memcpy(out, r, 32);
        } else if constexpr (BYTES == 16) {
            uint4 r = __ldg(reinterpret_cast<const uint4*>(p));
            memcpy(out, &r, 16);
        } else if constexpr (BYTES == 8) {
            uint2 r = __ldg(reinterpret_cast<const uint2*>(p));
            memcpy(out, &r, 8);
        } else {
            unsigned r = __ldg(reinterpret_cast<const unsigned*>(p));
            memcpy(out, &r, 4);
        }
    }
    __device__ __forceinline__ static void store(S* p, const S (&v)[V]) {
        if constexpr (BYTES == 32) {
            uint4 r[2];
            memcpy(r, v, 32);
            reinterpret_cast<uint4*>(p)[0] = r[0];
            reinterpret_cast<uint4*>(p)[1] = r[1];
        } else if constexpr (BYTES == 16) {
            uint4 r;
            memcpy(&r, v, 16);
            *reinterpret_cast<uint4*>(p) = r;
        } else if constexpr (BYTES == 8) {
            uint2 r;
            memcpy(&r, v, 8);
            *reinterpret_cast<uint2*>(p) = r;
        } else {
            unsigned r;
            memcpy(&r, v, 4);
            *reinterpret_cast<unsigned*>(p) = r;
        }
    }
};

// V solid bits (bit k <-> column xl + k) from V mask bytes that hold exactly
// 0 or 1: the multiply gathers byte k's low bit into bit 28 + k (every
// partial product lands on its own bit, so no carries interfere).
template <int V>
__device__ __forceinline__ uint32_t load_mask_core(const uint8_t* p) {
    constexpr uint32_t M = 0x10204080u;
    if constexpr (V == 8) {
        const uint2 r = __ldg(reinterpret_cast<const uint2*>(p));
        return ((r.x * M) >> 28) | (((r.y * M) >> 28) << 4);
    } else if constexpr (V == 4) {
        return (__ldg(reinterpret_cast<const unsigned*>(p)) * M) >> 28;
    } else if constexpr (V == 2) {
        return (uint32_t(__ldg(reinterpret_cast<const unsigned short*>(p))) * M) >> 28;
    } else {
        return __ldg(p);
    }
}

// Solid bit of column col of a mask row, with the x-axis rule for columns
// outside [0, w): wrapped when periodic, 0 otherwise (the axis rule decides).
__device__ __forceinline__ uint32_t mask_at(const uint8_t* row, int col, int w, bool xper) {
    if (col >= 0 && col < w) return __ldg(row + col);
    if (xper) {
        int c = col % w;
        if (c < 0) c += w;
        return __ldg(row + c);
    }
    return 0;
}

// Source row of a direction with row displacement dr; *cls = 0 (cells),
// 1 (zero-padded) or 2 (bounce-back wall) when the row lies outside.
__device__ __forceinline__ int source_row(int y, int dr, int h, int ym, int* cls) {
    int sr = y - dr;
    *cls = 0;
    if (sr < 0 || sr >= h) {
        if (ym == 1) sr = sr < 0 ? sr + h : sr - h;
        else { *cls = (ym == 2) ? 2 : 1; sr = 0; }
    }
    return sr;
}

// Collision of one cell in the reference's operation order (strict).
template <class CT>
__device__ __forceinline__ void collide_strict(const Consts<CT>& c, const CT (&f)[9],
                                               CT (&out)[9]) {
    using A = Ar<false>;
    // density (src/lbm.rs:117-121) and momentum_density (:123-131); the terms
    // f_i * 0 and the +-1 products are exact, so the nonzero terms are summed
    // in the reference's order.
    CT rho = A::add(CT(0), f[0]);
#pragma unroll
    for (int i = 1; i < 9; ++i) rho = A::add(rho, f[i]);
    CT mx = A::sub(f[1], f[3]);
    mx = A::add(mx, f[5]);
    mx = A::sub(mx, f[6]);
    mx = A::sub(mx, f[7]);
    mx = A::add(mx, f[8]);
    CT my = A::sub(f[2], f[4]);
    my = A::add(my, f[5]);
    my = A::add(my, f[6]);
    my = A::sub(my, f[7]);
    my = A::sub(my, f[8]);
    if (c.force) { mx = A::add(mx, c.hfx); my = A::add(my, c.hfy); }
    const CT inv = A::rcp(rho);                 // Matrix::recip (src/matrix.rs:133-136)
    const CT ux = A::mul(inv, mx);
    const CT uy = A::mul(inv, my);
    const CT v2k3 = A::mul(A::add(A::mul(ux, ux), A::mul(uy, uy)), c.k3);
    // c_i . u for each direction (exact negations of the reference's products).
    CT vc[9];
    vc[0] = CT(0);
    vc[1] = ux;
    vc[2] = uy;
    vc[3] = -ux;
    vc[4] = -uy;
    vc[5] = A::add(ux, uy);
    vc[6] = A::sub(uy, ux);
    vc[7] = -vc[5];
    vc[8] = A::sub(ux, uy);
    const CT rw0 = A::mul(rho, c.wt[0]);
    const CT rw1 = A::mul(rho, c.wt[1]);
    const CT rw5 = A::mul(rho, c.wt[5]);
    CT feq[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) {
        const CT rw = i == 0 ? rw0 : (i < 5 ? rw1 : rw5);
        CT s = A::add(CT(1), A::mul(vc[i], c.k1));
        s = A::add(s, A::mul(A::mul(vc[i], vc[i]), c.k2));
        s = A::add(s, v2k3);
        feq[i] = A::mul(rw, s);
    }
    if (c.collision == LBM_COLLISION_TRT) {
#pragma unroll
        for (int i = 0; i < 9; ++i) {
            const int o = OPP(i);
            const CT fsw = f[o];
            // swap_equilibrium fills entries 1..8 from the populations
            // (src/lbm.rs:311-322); kept as written.
            const CT eqsw = (i == 0) ? feq[0] : f[o];
            const CT fp = A::add(f[i], fsw);
            const CT fm = A::sub(f[i], fsw);
            const CT ep = A::add(feq[i], eqsw);
            const CT em = A::sub(feq[i], eqsw);
            const CT om = A::mul(A::add(A::mul(A::sub(fp, ep), c.omega_p),
                                        A::mul(A::sub(fm, em), c.omega_m)),
                                 c.trt_scale);
            out[i] = A::add(f[i], om);
        }
    } else {
#pragma unroll
        for (int i = 0; i < 9; ++i) out[i] = A::add(f[i], A::mul(A::sub(f[i], feq[i]), c.bgk_factor));
    }
    if (c.force) {
#pragma unroll
        for (int i = 0; i < 9; ++i) {
            const CT cx = CT(CX(i)), cy = CT(CY(i));
            const CT vci = A::add(A::mul(ux, cx), A::mul(uy, cy));
            const CT t1 = A::mul(A::add(A::mul(A::sub(cx, ux), c.fx),
                                        A::mul(A::sub(cy, uy), c.fy)), c.k1);
            const CT t2 = A::mul(A::mul(vci, A::add(A::mul(cx, c.fx), A::mul(cy, c.fy))),
                                 c.inv_cs4);
            const CT wg = A::mul(c.guo, c.wt[i]);
            out[i] = A::add(out[i], A::mul(wg, A::add(t1, t2)));
        }
    }
}

// The same collision with contracted, regrouped arithmetic: opposite
// directions share |c.u| so f_eq of a pair is A +- B, and the Guo term uses
// the precomputed c_i . F.
template <class CT>
__device__ __forceinline__ void collide_fast(const Consts<CT>& c, const CT (&f)[9],
                                             CT (&out)[9]) {
    const CT rho = ((f[0] + f[1]) + (f[2] + f[3])) + ((f[4] + f[5]) + (f[6] + f[7])) + f[8];
    CT mx = (f[1] - f[3]) + (f[5] - f[6]) + (f[8] - f[7]);
    CT my = (f[2] - f[4]) + (f[5] + f[6]) - (f[7] + f[8]);
    if (c.force) { mx += c.hfx; my += c.hfy; }
    const CT inv = Ar<true>::rcp(rho);
    const CT ux = mx * inv, uy = my * inv;
    const CT base = fma(fma(ux, ux, uy * uy), c.k3, CT(1));
    const CT rw0 = rho * c.wt[0], rw1 = rho * c.wt[1], rw5 = rho * c.wt[5];
    const CT rk1 = rw1 * c.k1, rk5 = rw5 * c.k1;
    CT feq[9];
    feq[0] = rw0 * base;
    {
        const CT A = rw1 * fma(c.k2, ux * ux, base), B = rk1 * ux;
        feq[1] = A + B; feq[3] = A - B;
    }
    {
        const CT A = rw1 * fma(c.k2, uy * uy, base), B = rk1 * uy;
        feq[2] = A + B; feq[4] = A - B;
    }
    const CT d = ux + uy, e = uy - ux;
    {
        const CT A = rw5 * fma(c.k2, d * d, base), B = rk5 * d;
        feq[5] = A + B; feq[7] = A - B;
    }
    {
        const CT A = rw5 * fma(c.k2, e * e, base), B = rk5 * e;
        feq[6] = A + B; feq[8] = A - B;
    }
    if (c.collision == LBM_COLLISION_TRT) {
#pragma unroll
        for (int i = 0; i < 9; ++i) {
            const CT fsw = f[OPP(i)];
            const CT eqsw = (i == 0) ? feq[0] : fsw;
            const CT om = ((f[i] + fsw) - (feq[i] + eqsw)) * c.omega_p +
                          ((f[i] - fsw) - (feq[i] - eqsw)) * c.omega_m;
            out[i] = fma(om, c.trt_scale, f[i]);
        }
    } else {
#pragma unroll
        for (int i = 0; i < 9; ++i) out[i] = fma(f[i] - feq[i], c.bgk_factor, f[i]);
    }
    if (c.force) {
        // S_i = guo w_i (k1 (c_i.F - u.F) + (c_i.u)(c_i.F)/cs^4)
        const CT uF = c.k1 * fma(ux, c.fx, uy * c.fy);
        CT vc[9];
        vc[0] = CT(0); vc[1] = ux; vc[2] = uy; vc[3] = -ux; vc[4] = -uy;
        vc[5] = d; vc[6] = e; vc[7] = -d; vc[8] = -e;
#pragma unroll
        for (int i = 0; i < 9; ++i)
            out[i] = fma(c.gw[i], fma(vc[i], c.cF4[i], c.kcF[i] - uF), out[i]);
    }
}

template <bool FAST, class CT>
__device__ __forceinline__ void collide_cell(const Consts<CT>& c, const CT (&f)[9], CT (&out)[9]) {
    if constexpr (FAST) collide_fast<CT>(c, f, out);
    else collide_strict<CT>(c, f, out);
}

// The same collision in the scaled deviation variables of 16-bit storage,
// G_i = s (f_i - w_i):  rho = 1 + sum(G)/s,  u = sum(G c)/(s + sum(G)),
// G_eq_i = w_i (sum(G) + (s + sum(G)) P_i) with P_i = k1 c.u + k2 (c.u)^2
// + k3 u^2, and BGK / Guo are linear in G.  No offset by w_i is ever added or
// removed, so loads and stores are bare format conversions.
template <class CT>
__device__ __forceinline__ void collide_dev(const Consts<CT>& c, const CT (&G)[9], CT (&out)[9]) {
    const CT DR = ((G[0] + G[1]) + (G[2] + G[3])) + ((G[4] + G[5]) + (G[6] + G[7])) + G[8];
    CT jx = (G[1] - G[3]) + (G[5] - G[6]) + (G[8] - G[7]);
    CT jy = (G[2] - G[4]) + (G[5] + G[6]) - (G[7] + G[8]);
    if (c.force) { jx += c.shfx; jy += c.shfy; }
    const CT RS = c.dscale + DR;                          // s * rho
    const CT inv = Ar<true>::rcp(RS);
    const CT ux = jx * inv, uy = jy * inv;
    const CT u2k3 = c.k3 * fma(ux, ux, uy * uy);
    const CT rs0 = RS * c.wt[0], rs1 = RS * c.wt[1], rs5 = RS * c.wt[5];
    const CT wd0 = DR * c.wt[0], wd1 = DR * c.wt[1], wd5 = DR * c.wt[5];
    CT geq[9];
    geq[0] = fma(rs0, u2k3, wd0);
    {
        const CT A = fma(c.k2, ux * ux, u2k3), B = c.k1 * ux;
        geq[1] = fma(rs1, A + B, wd1); geq[3] = fma(rs1, A - B, wd1);
    }
    {
        const CT A = fma(c.k2, uy * uy, u2k3), B = c.k1 * uy;
        geq[2] = fma(rs1, A + B, wd1); geq[4] = fma(rs1, A - B, wd1);
    }
    const CT d = ux + uy, e = uy - ux;
    {
        const CT A = fma(c.k2, d * d, u2k3), B = c.k1 * d;
        geq[5] = fma(rs5, A + B, wd5); geq[7] = fma(rs5, A - B, wd5);
    }
    {
        const CT A = fma(c.k2, e * e, u2k3), B = c.k1 * e;
        geq[6] = fma(rs5, A + B, wd5); geq[8] = fma(rs5, A - B, wd5);
    }
    if (c.collision == LBM_COLLISION_TRT) {
#pragma unroll
        for (int i = 0; i < 9; ++i) {
            const CT gsw = G[OPP(i)];
            const CT eqsw = (i == 0) ? geq[0] : gsw;
            const CT om = ((G[i] + gsw) - (geq[i] + eqsw)) * c.omega_p +
                          ((G[i] - gsw) - (geq[i] - eqsw)) * c.omega_m;
            out[i] = fma(om, c.trt_scale, G[i]);
        }
    } else {
#pragma unroll
        for (int i = 0; i < 9; ++i) out[i] = fma(G[i] - geq[i], c.bgk_factor, G[i]);
    }
    if (c.force) {
        const CT uF = c.k1 * fma(ux, c.fx, uy * c.fy);
        CT vc[9];
        vc[0] = CT(0); vc[1] = ux; vc[2] = uy; vc[3] = -ux; vc[4] = -uy;
        vc[5] = d; vc[6] = e; vc[7] = -d; vc[8] = -e;
#pragma unroll
        for (int i = 0; i < 9; ++i)
            out[i] = fma(c.sgw[i], fma(vc[i], c.cF4[i], c.kcF[i] - uF), out[i]);
    }
}

// Moments of a stored cell state (Lattice::density / velocity, src/lbm.rs:
// 117-149), with u = (j - F/2)/rho when a body force is set.
template <bool FAST, class CT>
__device__ __forceinline__ void cell_moments(const Consts<CT>& c, const CT (&f)[9],
                                             CT& rho, CT& ux, CT& uy) {
    using A = Ar<FAST>;
    rho = A::add(CT(0), f[0]);
#pragma unroll
    for (int i = 1; i < 9; ++i) rho = A::add(rho, f[i]);
    CT mx = A::sub(f[1], f[3]);
    mx = A::add(mx, f[5]);
    mx = A::sub(mx, f[6]);
    mx = A::sub(mx, f[7]);
    mx = A::add(mx, f[8]);
    CT my = A::sub(f[2], f[4]);
    my = A::add(my, f[5]);
    my = A::add(my, f[6]);
    my = A::sub(my, f[7]);
    my = A::sub(my, f[8]);
    if (c.force) { mx = A::sub(mx, c.hfx); my = A::sub(my, c.hfy); }
    const CT inv = A::rcp(rho);
    ux = A::mul(inv, mx);
    uy = A::mul(inv, my);
}

// Moments of a stored cell given in the step kernels' working variables.
template <class S, bool FAST, class CT>
__device__ __forceinline__ void domain_moments(const Consts<CT>& c, const CT (&g)[9], CT& rho,
                                               CT& ux, CT& uy) {
    if constexpr (Store<S>::DEV) {
        const CT DR = ((g[0] + g[1]) + (g[2] + g[3])) + ((g[4] + g[5]) + (g[6] + g[7])) + g[8];
        CT jx = (g[1] - g[3]) + (g[5] - g[6]) + (g[8] - g[7]);
        CT jy = (g[2] - g[4]) + (g[5] + g[6]) - (g[7] + g[8]);
        if (c.force) { jx -= c.shfx; jy -= c.shfy; }
        const CT inv = Ar<true>::rcp(c.dscale + DR);
        rho = CT(1) + DR * c.dinv;
        ux = jx * inv;
        uy = jy * inv;
    } else {
        cell_moments<FAST>(c, g, rho, ux, uy);
    }
}

// The collision in the working variables of storage type S.
template <class S, bool FAST, class CT>
__device__ __forceinline__ void collide_domain(const Consts<CT>& c, const CT (&g)[9], CT (&out)[9]) {
    if constexpr (Store<S>::DEV) collide_dev<CT>(c, g, out);
    else collide_cell<FAST>(c, g, out);
}

// Collides a thread's V cells in place.  f32 collision arithmetic in fast or
// deviation form takes the cells in pairs on the packed f32x2 instructions.
#ifndef LBM_PAIRED
#define LBM_PAIRED 1
#endif
template <class S, int V, bool FAST>
__device__ __forceinline__ void collide_cells(const Consts<typename Store<S>::CT>& c,
                                              typename Store<S>::CT (&f)[9][V]) {
    using CT = typename Store<S>::CT;
    constexpr bool paired = LBM_PAIRED && sizeof(CT) == 4 && V % 2 == 0 && (FAST || Store<S>::DEV);
    if constexpr (paired) {
#pragma unroll
        for (int k = 0; k < V; k += 2) {
            float2 g[9], o[9];
#pragma unroll
            for (int i = 0; i < 9; ++i) g[i] = make_float2(f[i][k], f[i][k + 1]);
            if constexpr (Store<S>::DEV) collide_dev_x2(c, g, o);
            else collide_fast_x2(c, g, o);
#pragma unroll
            for (int i = 0; i < 9; ++i) { f[i][k] = o[i].x; f[i][k + 1] = o[i].y; }
        }
    } else {
#pragma unroll
        for (int k = 0; k < V; ++k) {
            CT g[9], o[9];
#pragma unroll
            for (int i = 0; i < 9; ++i) g[i] = f[i][k];
            collide_domain<S, FAST>(c, g, o);
#pragma unroll
            for (int i = 0; i < 9; ++i) f[i][k] = o[i];
        }
    }
}

// Writes the V collided cells of a thread and, when requested, their moments
// (computed from the stored, i.e. encoded, values).
template <class S, int V, bool FAST, class A>
__device__ __forceinline__ void store_cells(const A& a, int y,
                                            int x0, const S (&enc)[9][V]) {
    using CT = typename Store<S>::CT;
    using ST = Store<S>;
    S* __restrict__ dst = static_cast<S*>(a.dst);
    const int64_t PL = a.plane;
    const int w = a.w;
    const int64_t base = int64_t(y) * a.pitch + x0;
    if (x0 + V <= w) {
#pragma unroll
        for (int i = 0; i < 9; ++i) VecIO<S, V>::store(dst + i * PL + base, enc[i]);
    } else {
#pragma unroll
        for (int i = 0; i < 9; ++i)
#pragma unroll
            for (int k = 0; k < V; ++k)
                if (x0 + k < w) dst[i * PL + base + k] = enc[i][k];
    }
    if (a.mom_rho != nullptr) {
        const int64_t mbase = int64_t(y) * a.mom_pitch + x0;
        float mr[V], mx[V], my[V];
#pragma unroll
        for (int k = 0; k < V; ++k) {
            CT g[9];
#pragma unroll
            for (int i = 0; i < 9; ++i) g[i] = ST::dec_dom(enc[i][k]);
            CT r, ux, uy;
            domain_moments<S, FAST>(a.c, g, r, ux, uy);
            mr[k] = float(r);
            mx[k] = float(ux);
            my[k] = float(uy);
        }
        // whole, 16-byte aligned runs go out as vectors (the outputs may be
        // host memory written over the host link, where wide writes matter)
        if constexpr (V % 4 == 0) {
            const bool aligned = ((reinterpret_cast<uintptr_t>(a.mom_rho) |
                                   reinterpret_cast<uintptr_t>(a.mom_ux) |
                                   reinterpret_cast<uintptr_t>(a.mom_uy)) & 15u) == 0;
            if (aligned && x0 + V <= w && (mbase & 3) == 0) {
#pragma unroll
                for (int k = 0; k < V; k += 4) {
                    *reinterpret_cast<float4*>(a.mom_rho + mbase + k) = make_float4(mr[k], mr[k + 1], mr[k + 2], mr[k + 3]);
                    *reinterpret_cast<float4*>(a.mom_ux + mbase + k) = make_float4(mx[k], mx[k + 1], mx[k + 2], mx[k + 3]);
                    *reinterpret_cast<float4*>(a.mom_uy + mbase + k) = make_float4(my[k], my[k + 1], my[k + 2], my[k + 3]);
                }
                return;
            }
        }
#pragma unroll
        for (int k = 0; k < V; ++k) {
            if (x0 + k >= w) break;
            a.mom_rho[mbase + k] = mr[k];
            a.mom_ux[mbase + k] = mx[k];
            a.mom_uy[mbase + k] = my[k];
        }
    }
}

// L2 prefetch ahead of the wavefront: blocks run in row-major order, so the
// rows that the warp a.pf_rows rows further down will pull are fetched into
// L2 now (one bulk prefetch of the warp's 32 V columns per plane, lanes 0-8)
// and that warp's loads find them there.  Interior tiles only (full tiles, so
// the range stays inside the row).
template <class S, int V, int FRAME, class A>
__device__ __forceinline__ void prefetch_ahead(const A& a, int y, int x0, int lane) {
    if (a.pf_rows > 0 && lane < 9) {
        const int ys = y + a.pf_rows - DROW(FRAME, lane);
        if (ys < a.h) {
            const S* p = static_cast<const S*>(a.src) + lane * a.plane + int64_t(ys) * a.pitch +
                         (x0 - lane * V);
            asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;"
                         :: "l"(p), "n"(32 * V * int(sizeof(S))) : "memory");
        }
    }
}

// 16-bit storage with stochastic rounding: the cells of a partial last chunk
// that lie past the lattice edge collide zeros.  A stored cell's rounding
// hashes its pair partner too, so the partner must not depend on which path
// loaded it.
template <class S, int V>
__device__ __forceinline__ void zero_past_edge(typename Store<S>::CT (&f)[9][V], int x0, int w) {
#pragma unroll
    for (int i = 0; i < 9; ++i)
#pragma unroll
        for (int k = 0; k < V; ++k)
            if (x0 + k >= w) f[i][k] = 0;
}

// Source rows and warp-edge columns of an interior tile.  Rows wrap at the
// y edges and columns at the x edges: an interior tile reaches an edge only
// when that axis is periodic (tiles at other edges are listed), so the wrap
// is always the right rule.
struct InteriorRows {
    int64_t rm, r0, rp;     // element offsets of rows y - 1, y, y + 1
    int left, right;        // columns x0 - 1 and x0 + V, wrapped
    template <class A>
    __device__ __forceinline__ InteriorRows(const A& a, int y, int x0, int V) {
        const int64_t P = a.pitch;
        rm = int64_t(y == 0 ? a.h - 1 : y - 1) * P;
        r0 = int64_t(y) * P;
        rp = int64_t(y == a.h - 1 ? 0 : y + 1) * P;
        left = x0 == 0 ? a.w - 1 : x0 - 1;
        right = x0 + V == a.w ? 0 : x0 + V;
    }
    // offset of the source row of a direction with row displacement dr
    __device__ __forceinline__ int64_t of(int dr) const { return dr == 1 ? rm : (dr == -1 ? rp : r0); }
};

// Interior warp tile (flag 0): every source cell is inside the lattice and
// fluid, so a step is 9 vector loads, 6 shuffles and two edge scalars per
// lane, the collision and 9 vector stores.  With GEN_CT (a tile flagged 3 of
// a lattice with link masks: solids nearby, no lattice edge in reach) the
// same code applies the fixups of step_general from the tile's per-lane link
// masks: bounce-back links take the cell's own opposite population, solid
// cells swap (full-way) or keep their populations (half-way).
template <class S, int V, int FRAME, bool FAST, bool SR = false, bool GEN_CT = false, class A>
__device__ __forceinline__ void step_interior(const A& a, int y,
                                              int x0, int lane, int tile = 0) {
    using CT = typename Store<S>::CT;
    using ST = Store<S>;
    const S* __restrict__ src = static_cast<const S*>(a.src);
    const int64_t PL = a.plane;
    const InteriorRows rows(a, y, x0, V);
    uint4 lk = make_uint4(0u, 0u, 0u, 0u);
    if constexpr (GEN_CT) lk = __ldg(a.links + (int64_t(y) * a.ntiles + tile) * 32 + lane);
    S raw[9][V];
    S edge[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) {
        const int dc = DCOL(FRAME, i), dr = DROW(FRAME, i);
        const S* prow = src + i * PL + rows.of(dr);
        VecIO<S, V>::load(prow + x0, raw[i]);
        edge[i] = raw[i][0];
        if (dc == 1 && lane == 0) edge[i] = __ldg(prow + rows.left);
        if (dc == -1 && lane == 31) edge[i] = __ldg(prow + rows.right);
    }
    prefetch_ahead<S, V, FRAME>(a, y, x0, lane);
    CT f[9][V];
#pragma unroll
    for (int i = 0; i < 9; ++i) {
        const int dc = DCOL(FRAME, i);
        CT v[V];
        ST::dec_vec_dom(raw[i], v);
        if (dc == 1) {
            const CT left = __shfl_up_sync(kFull, v[V - 1], 1);
#pragma unroll
            for (int k = V - 1; k > 0; --k) v[k] = v[k - 1];
            v[0] = lane == 0 ? ST::dec_dom(edge[i]) : left;
        } else if (dc == -1) {
            const CT right = __shfl_down_sync(kFull, v[0], 1);
#pragma unroll
            for (int k = 0; k < V - 1; ++k) v[k] = v[k + 1];
            v[V - 1] = lane == 31 ? ST::dec_dom(edge[i]) : right;
        }
#pragma unroll
        for (int k = 0; k < V; ++k) f[i][k] = v[k];
    }
    constexpr uint32_t FULL = (1u << V) - 1u;
    const uint32_t own_solid = GEN_CT ? (lk.x & FULL) : 0u;
    const bool halfway = (a.flags & LBM_SOLID_HALFWAY) != 0;
    if constexpr (GEN_CT) {
        const uint32_t words[3] = {lk.x, lk.y, lk.z};
#pragma unroll
        for (int i = 1; i < 9; ++i) {
            const uint32_t bnc = (words[i >> 2] >> (8 * (i & 3))) & FULL;
            if (bnc) {
                S own[V];
                VecIO<S, V>::load(src + OPP(i) * PL + rows.r0 + x0, own);
#pragma unroll
                for (int k = 0; k < V; ++k)
                    if ((bnc >> k) & 1u) f[i][k] = ST::dec_dom(own[k]);
            }
        }
        if (own_solid && !halfway) {
            // bounce_back (src/lbm.rs:741-751): solid nodes take swapped populations
#pragma unroll
            for (int k = 0; k < V; ++k) {
                if ((own_solid >> k) & 1u) {
                    CT t;
                    t = f[1][k]; f[1][k] = f[3][k]; f[3][k] = t;
                    t = f[2][k]; f[2][k] = f[4][k]; f[4][k] = t;
                    t = f[5][k]; f[5][k] = f[7][k]; f[7][k] = t;
                    t = f[6][k]; f[6][k] = f[8][k]; f[8][k] = t;
                }
            }
        }
    }
    collide_cells<S, V, FAST>(a.c, f);
    S enc[9][V];
#pragma unroll
    for (int i = 0; i < 9; ++i) ST::enc_vec_dom(f[i], enc[i], SR ? 1 : 0);
    if (GEN_CT && own_solid && halfway) {
        // half-way mode: solid nodes keep their populations
#pragma unroll
        for (int i = 0; i < 9; ++i) {
            S own[V];
            VecIO<S, V>::load(src + i * PL + rows.r0 + x0, own);
#pragma unroll
            for (int k = 0; k < V; ++k)
                if ((own_solid >> k) & 1u) enc[i][k] = own[k];
        }
    }
    store_cells<S, V, FAST>(a, y, x0, enc);
}

// One time step of one lattice.  Phase A issues every global load of the
// thread (3 mask rows, 9 population vectors and the warp-edge scalars) before
// any of them is consumed, so a thread has ~150 B in flight and pays one
// memory latency; phase B realigns the +-1 column shifts with shuffles and
// classifies boundary links; phase C fetches the cell's own opposite
// populations for bounce-back links (only near walls and solids); phase D
// collides and stores.
// Periodic-edge warp tile (flag 2): the partial last tile of a row of a
// lattice periodic in x (full tiles at periodic edges take the interior
// path, which wraps rows and its edge columns).  Every source cell is fluid.
// A step is 9 vector loads, 6 shuffles, two edge scalars per lane, the
// collision and 9 vector stores; the edge rows and columns wrap.  Lanes past
// the edge only feed the shuffles, and the lane holding column w - 1 takes
// column 0 for the cell whose source lies past the edge.
template <class S, int V, int FRAME, bool FAST, bool SR = false, class A>
__device__ __forceinline__ void step_interior_wrap(const A& a, int y,
                                              int x0, int lane) {
    using CT = typename Store<S>::CT;
    using ST = Store<S>;
    const int w = a.w, h = a.h;
    const int64_t P = a.pitch, PL = a.plane;
    const S* __restrict__ src = static_cast<const S*>(a.src);
    const int ym1 = y == 0 ? h - 1 : y - 1, yp1 = y == h - 1 ? 0 : y + 1;
    const int xl = x0 < w ? x0 : 0;                 // idle lanes read a valid chunk
    const bool last = x0 < w && x0 + V >= w;        // this chunk holds column w - 1
    S raw[9][V];
    S edge[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) {
        const int dc = DCOL(FRAME, i), dr = DROW(FRAME, i);
        const int sr = dr == 1 ? ym1 : (dr == -1 ? yp1 : y);
        const S* prow = src + i * PL + int64_t(sr) * P;
        VecIO<S, V>::load(prow + xl, raw[i]);
        edge[i] = raw[i][0];
        if (dc == 1 && lane == 0) edge[i] = __ldg(prow + (x0 == 0 ? w - 1 : x0 - 1));
        if (dc == -1) {
            if (last) edge[i] = __ldg(prow);               // column w wraps to 0
            else if (lane == 31 && x0 < w) edge[i] = __ldg(prow + x0 + V);
        }
    }
    CT f[9][V];
#pragma unroll
    for (int i = 0; i < 9; ++i) {
        const int dc = DCOL(FRAME, i);
        CT v[V];
        ST::dec_vec_dom(raw[i], v);
        if (dc == 1) {
            const CT left = __shfl_up_sync(kFull, v[V - 1], 1);
#pragma unroll
            for (int k = V - 1; k > 0; --k) v[k] = v[k - 1];
            v[0] = lane == 0 ? ST::dec_dom(edge[i]) : left;
        } else if (dc == -1) {
            const CT right = __shfl_down_sync(kFull, v[0], 1);
#pragma unroll
            for (int k = 0; k < V - 1; ++k) v[k] = v[k + 1];
            const CT e = ST::dec_dom(edge[i]);
            v[V - 1] = lane == 31 ? e : right;
            if (last) {
#pragma unroll
                for (int k = 0; k < V; ++k)
                    if (x0 + k == w - 1) v[k] = e;
            }
        }
#pragma unroll
        for (int k = 0; k < V; ++k) f[i][k] = v[k];
    }
    if (SR && last) zero_past_edge<S, V>(f, x0, w);
    collide_cells<S, V, FAST>(a.c, f);
    S enc[9][V];
#pragma unroll
    for (int i = 0; i < 9; ++i) ST::enc_vec_dom(f[i], enc[i], SR ? 1 : 0);
    if (x0 < w) store_cells<S, V, FAST>(a, y, x0, enc);
}

// 16-bit storage keeps a thread's values packed two per register (element
// 2j in the low half of register j) until the collision: the +-1 column
// shifts become one byte permute per register, and only one cell pair is
// widened to f32 at a time, so the working set stays small enough for V = 8.
template <int NP>
struct PackIO {
    __device__ __forceinline__ static void load(const void* p, uint32_t (&r)[NP]) {
        if constexpr (NP == 4) {
            const uint4 q = __ldg(reinterpret_cast<const uint4*>(p));
            r[0] = q.x; r[1] = q.y; r[2] = q.z; r[3] = q.w;
        } else {
            static_assert(NP == 2, "4 or 8 cells per thread");
            const uint2 q = __ldg(reinterpret_cast<const uint2*>(p));
            r[0] = q.x; r[1] = q.y;
        }
    }
    __device__ __forceinline__ static void store(void* p, const uint32_t (&r)[NP]) {
        if constexpr (NP == 4) *reinterpret_cast<uint4*>(p) = make_uint4(r[0], r[1], r[2], r[3]);
        else *reinterpret_cast<uint2*>(p) = make_uint2(r[0], r[1]);
    }
};

// Pull shift by one column toward higher x (c_x = +1 in the row direction):
// element k takes element k - 1; `left` holds the value entering at k = 0 in
// its high half.
template <int NP>
__device__ __forceinline__ void shift_up_packed(uint32_t (&r)[NP], uint32_t left) {
#pragma unroll
    for (int j = NP - 1; j > 0; --j) r[j] = __byte_perm(r[j - 1], r[j], 0x5432);
    r[0] = __byte_perm(left, r[0], 0x5432);
}
// Element k takes element k + 1; `right` holds the value entering at the top
// in its low half.
template <int NP>
__device__ __forceinline__ void shift_down_packed(uint32_t (&r)[NP], uint32_t right) {
#pragma unroll
    for (int j = 0; j < NP - 1; ++j) r[j] = __byte_perm(r[j], r[j + 1], 0x5432);
    r[NP - 1] = __byte_perm(r[NP - 1], right, 0x5432);
}
// Replaces element k of a packed row by the 16-bit value e.
template <int NP>
__device__ __forceinline__ void set_packed(uint32_t (&r)[NP], int k, uint32_t e) {
#pragma unroll
    for (int j = 0; j < NP; ++j) {
        if (k == 2 * j) r[j] = (r[j] & 0xffff0000u) | (e & 0xffffu);
        else if (k == 2 * j + 1) r[j] = (r[j] & 0xffffu) | (e << 16);
    }
}

// Collides the pairs of a packed 16-bit tile in place.  Every pair is
// widened, collided by collide_dev_x2 and narrowed exactly as collide_cells +
// enc_vec_dom do, so the results are the same bits as the unpacked path's.
// With SUB (general tiles), zero-padded links (bit k of zb[i]) take the
// deviation value of f = 0 after widening, and cells past the lattice edge
// (bit k of past) collide zeros under stochastic rounding (zero_past_edge).
// With ROLL the pairs are taken in a loop that is not unrolled: each pass
// collides register 0 of every plane and rotates the registers down, so the
// collision's code appears once (the general paths, where code size and not
// the rotation's moves is what costs).
template <class S, int V, bool SR, bool SUB = false, bool ROLL = false>
__device__ __forceinline__ void collide_packed(const Consts<float>& c, uint32_t (&r)[9][V / 2],
                                               const uint32_t* zb = nullptr, uint32_t past = 0u) {
    using ST = Store<S>;
    using H2 = decltype(ST::from_f2(make_float2(0.f, 0.f)));
    constexpr int NP = V / 2;
    uint32_t any = SR ? past : 0u;                 // cells that take a substitute
    if constexpr (SUB) {
#pragma unroll
        for (int i = 0; i < 9; ++i) any |= zb[i];
    }
    if constexpr (ROLL) {
        uint32_t zl[9];
#pragma unroll
        for (int i = 0; i < 9; ++i) zl[i] = SUB ? zb[i] : 0u;
        uint32_t pl = past;
#pragma unroll 1
        for (int j = 0; j < NP; ++j) {
            float2 g[9], o[9];
#pragma unroll
            for (int i = 0; i < 9; ++i) {
                H2 p;
                memcpy(&p, &r[i][0], 4);
                g[i] = ST::to_f2(p);
            }
            if (SUB && (any & 3u)) {
#pragma unroll
                for (int i = 0; i < 9; ++i) {
                    const float zv = ST::zero_dom(c.wt[i], c.dscale);
                    if (zl[i] & 1u) g[i].x = zv;
                    if (zl[i] & 2u) g[i].y = zv;
                    if (SR && (pl & 1u)) g[i].x = 0.f;
                    if (SR && (pl & 2u)) g[i].y = 0.f;
                }
            }
            collide_dev_x2(c, g, o);
#pragma unroll
            for (int i = 0; i < 9; ++i) {
                const H2 p = SR ? ST::from_f2_sr(o[i].x, o[i].y) : ST::from_f2(o[i]);
#pragma unroll
                for (int k = 0; k < NP - 1; ++k) r[i][k] = r[i][k + 1];
                memcpy(&r[i][NP - 1], &p, 4);
                zl[i] >>= 2;
            }
            pl >>= 2;
            any >>= 2;
        }
        return;
    }
#pragma unroll
    for (int j = 0; j < NP; ++j) {
        float2 g[9], o[9];
#pragma unroll
        for (int i = 0; i < 9; ++i) {
            H2 p;
            memcpy(&p, &r[i][j], 4);
            g[i] = ST::to_f2(p);
        }
        if (SUB && ((any >> (2 * j)) & 3u)) {
#pragma unroll
            for (int i = 0; i < 9; ++i) {
                const uint32_t z = zb[i] >> (2 * j);
                const float zv = ST::zero_dom(c.wt[i], c.dscale);
                if (z & 1u) g[i].x = zv;
                if (z & 2u) g[i].y = zv;
                if (SR && ((past >> (2 * j)) & 1u)) g[i].x = 0.f;
                if (SR && ((past >> (2 * j)) & 2u)) g[i].y = 0.f;
            }
        }
        collide_dev_x2(c, g, o);
#pragma unroll
        for (int i = 0; i < 9; ++i) {
            const H2 p = SR ? ST::from_f2_sr(o[i].x, o[i].y) : ST::from_f2(o[i]);
            memcpy(&r[i][j], &p, 4);
        }
    }
}

// Writes a packed tile's cells of row y from column x0 (and the moments when
// requested).
template <class S, int V>
__device__ __forceinline__ void store_packed(const StepArgs<float>& a, int y, int x0,
                                             const uint32_t (&r)[9][V / 2]) {
    constexpr int NP = V / 2;
    if (x0 + V <= a.w && a.mom_rho == nullptr) {
        S* __restrict__ dst = static_cast<S*>(a.dst) + int64_t(y) * a.pitch + x0;
#pragma unroll
        for (int i = 0; i < 9; ++i) PackIO<NP>::store(dst + i * a.plane, r[i]);
        return;
    }
    S enc[9][V];
#pragma unroll
    for (int i = 0; i < 9; ++i) memcpy(enc[i], r[i], sizeof(enc[i]));
    store_cells<S, V, true>(a, y, x0, enc);
}

template <class S, int V, bool SR, bool ROLL = false>
__device__ __forceinline__ void collide_store_packed(const StepArgs<float>& a, int y, int x0,
                                                     uint32_t (&r)[9][V / 2]) {
    collide_packed<S, V, SR, false, ROLL>(a.c, r);
    store_packed<S, V>(a, y, x0, r);
}

// Mask of the 16-bit halves of register j selected by bits 2j, 2j + 1 of b.
__device__ __forceinline__ uint32_t half_mask(uint32_t b, int j) {
    return (((b >> (2 * j)) & 1u) ? 0x0000ffffu : 0u) | (((b >> (2 * j + 1)) & 1u) ? 0xffff0000u : 0u);
}

// Tiles flagged 3 run a second instantiation of the interior code (GEN):
// with LBM_GEN_OWN it loads the cells' own populations up front, with
// LBM_ROLL_GEN its pair loop is rolled (fewer registers: the unrolled form
// spilled).  A/B on one GB300, 4096^2 channel, 16-bit stochastic: fixups as a
// run-time branch of the interior code 149.0k MLUPS (the branch also slowed
// the pure interior path 4%); separate instantiation 151.4k; + own loads
// 152.4k; + rolled 153.8k; both 154.8k.
#ifndef LBM_GEN_OWN
#define LBM_GEN_OWN 1
#endif
#ifndef LBM_ROLL_GEN
#define LBM_ROLL_GEN 1
#endif
// Interior warp tile (flag 0) of 16-bit storage, packed.  With GEN_CT (a tile
// flagged 3 of a lattice with link masks: solids nearby, no lattice edge in
// reach) the same code runs with the fixups of step_general_packed, read from
// the tile's precomputed per-lane link masks instead of the mask rows:
// bounce-back links take the cell's own opposite population, and solid cells
// are swapped (full-way) or keep their populations (half-way).
template <class S, int V, int FRAME, bool SR, bool GEN_CT = false>
__device__ __forceinline__ void step_interior_packed(const StepArgs<float>& a, int y, int x0,
                                                     int lane, int tile = 0) {
    constexpr bool gen = GEN_CT;
    constexpr int NP = V / 2;
    constexpr uint32_t FULL = (1u << V) - 1u;
    const unsigned short* __restrict__ src = static_cast<const unsigned short*>(a.src);
    const int64_t PL = a.plane;
    const InteriorRows rows(a, y, x0, V);
    uint4 lk = make_uint4(0u, 0u, 0u, 0u);
    if (V == 8 && gen) lk = __ldg(a.links + (int64_t(y) * a.ntiles + tile) * 32 + lane);
    uint32_t r[9][NP];
    uint32_t edge[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) {
        const int dc = DCOL(FRAME, i), dr = DROW(FRAME, i);
        const unsigned short* prow = src + i * PL + rows.of(dr);
        PackIO<NP>::load(prow + x0, r[i]);
        edge[i] = 0u;
        if (dc == 1 && lane == 0) edge[i] = uint32_t(__ldg(prow + rows.left)) << 16;
        if (dc == -1 && lane == 31) edge[i] = __ldg(prow + rows.right);
    }
    // LBM_GEN_OWN: tiles flagged 3 load the cell's own populations (row y of
    // every plane) with everything else, so the bounce-back links and the
    // half-way keep need no second and third memory round trip; planes
    // without a row shift take them from their load before the column shift.
    uint32_t own[9][NP];
    if constexpr (LBM_GEN_OWN && GEN_CT && V == 8) {
#pragma unroll
        for (int i = 0; i < 9; ++i) {
            if (DROW(FRAME, i) != 0) PackIO<NP>::load(src + i * PL + rows.r0 + x0, own[i]);
            else {
#pragma unroll
                for (int j = 0; j < NP; ++j) own[i][j] = r[i][j];
            }
        }
    }
    prefetch_ahead<S, V, FRAME>(a, y, x0, lane);
#pragma unroll
    for (int i = 0; i < 9; ++i) {
        const int dc = DCOL(FRAME, i);
        if (dc == 1) {
            const uint32_t left = __shfl_up_sync(kFull, r[i][NP - 1], 1);
            shift_up_packed<NP>(r[i], lane == 0 ? edge[i] : left);
        } else if (dc == -1) {
            const uint32_t right = __shfl_down_sync(kFull, r[i][0], 1);
            shift_down_packed<NP>(r[i], lane == 31 ? edge[i] : right);
        }
    }
    uint32_t own_solid = 0u;
    const bool halfway = (a.flags & LBM_SOLID_HALFWAY) != 0;
    if (V == 8 && gen) {
        own_solid = lk.x & FULL;
        const uint32_t words[3] = {lk.x, lk.y, lk.z};
        // bounce-back links take the cell's own opposite population
#pragma unroll
        for (int i = 1; i < 9; ++i) {
            const uint32_t bnc = (words[i >> 2] >> (8 * (i & 3))) & FULL;
            if (bnc) {
                uint32_t ld[NP];
                if constexpr (LBM_GEN_OWN && GEN_CT) {
#pragma unroll
                    for (int j = 0; j < NP; ++j) ld[j] = own[OPP(i)][j];
                } else {
                    PackIO<NP>::load(src + OPP(i) * PL + rows.r0 + x0, ld);
                }
#pragma unroll
                for (int j = 0; j < NP; ++j) {
                    const uint32_t m = half_mask(bnc, j);
                    r[i][j] = (r[i][j] & ~m) | (ld[j] & m);
                }
            }
        }
        if (own_solid && !halfway) {
            // bounce_back (src/lbm.rs:741-751): solid nodes take swapped populations
#pragma unroll
            for (int p = 0; p < 4; ++p) {
                const int i0 = p < 2 ? 1 + p : 5 + (p - 2), i1 = OPP(i0);
#pragma unroll
                for (int j = 0; j < NP; ++j) {
                    const uint32_t m = half_mask(own_solid, j);
                    const uint32_t t = (r[i0][j] ^ r[i1][j]) & m;
                    r[i0][j] ^= t;
                    r[i1][j] ^= t;
                }
            }
        }
    }
    collide_packed<S, V, SR, false,
                   (V / 2 >= 4) && (GEN_CT ? LBM_ROLL_GEN : LBM_ROLL_INTERIOR)>(a.c, r);
    if (V == 8 && gen && own_solid && halfway) {
        // half-way mode: solid nodes keep their populations
#pragma unroll
        for (int i = 0; i < 9; ++i) {
            uint32_t ld[NP];
            if constexpr (LBM_GEN_OWN && GEN_CT) {
#pragma unroll
                for (int j = 0; j < NP; ++j) ld[j] = own[i][j];
            } else {
                PackIO<NP>::load(src + i * PL + rows.r0 + x0, ld);
            }
#pragma unroll
            for (int j = 0; j < NP; ++j) {
                const uint32_t m = half_mask(own_solid, j);
                r[i][j] = (r[i][j] & ~m) | (ld[j] & m);
            }
        }
    }
    store_packed<S, V>(a, y, x0, r);
}

// Periodic-edge warp tile (flag 2) of 16-bit storage, packed (the rules of
// step_interior_wrap).
template <class S, int V, int FRAME, bool SR>
__device__ __forceinline__ void step_interior_wrap_packed(const StepArgs<float>& a, int y, int x0,
                                                          int lane) {
    constexpr int NP = V / 2;
    const int w = a.w, h = a.h;
    const int64_t P = a.pitch, PL = a.plane;
    const S* __restrict__ src = static_cast<const S*>(a.src);
    const int ym1 = y == 0 ? h - 1 : y - 1, yp1 = y == h - 1 ? 0 : y + 1;
    const int xl = x0 < w ? x0 : 0;
    const bool last = x0 < w && x0 + V >= w;
    uint32_t r[9][NP];
    uint32_t edge[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) {
        const int dc = DCOL(FRAME, i), dr = DROW(FRAME, i);
        const int sr = dr == 1 ? ym1 : (dr == -1 ? yp1 : y);
        const unsigned short* prow =
            reinterpret_cast<const unsigned short*>(src + i * PL + int64_t(sr) * P);
        PackIO<NP>::load(prow + xl, r[i]);
        edge[i] = 0u;
        if (dc == 1 && lane == 0) edge[i] = uint32_t(__ldg(prow + (x0 == 0 ? w - 1 : x0 - 1))) << 16;
        if (dc == -1) {
            if (last) edge[i] = __ldg(prow);                  // column w wraps to 0
            else if (lane == 31 && x0 < w) edge[i] = __ldg(prow + x0 + V);
        }
    }
#pragma unroll
    for (int i = 0; i < 9; ++i) {
        const int dc = DCOL(FRAME, i);
        if (dc == 1) {
            const uint32_t left = __shfl_up_sync(kFull, r[i][NP - 1], 1);
            shift_up_packed<NP>(r[i], lane == 0 ? edge[i] : left);
        } else if (dc == -1) {
            const uint32_t right = __shfl_down_sync(kFull, r[i][0], 1);
            shift_down_packed<NP>(r[i], lane == 31 ? edge[i] : right);
            if (last) set_packed<NP>(r[i], w - 1 - x0, edge[i]);
        }
    }
    if (x0 >= w) return;                 // lanes past the edge only fed the shuffles
    if (SR && x0 + V > w) {
        // cells past the edge collide zeros: a stored cell's stochastic
        // rounding hashes its pair partner too, which must not depend on
        // the path that ran
#pragma unroll
        for (int i = 0; i < 9; ++i)
#pragma unroll
            for (int k = 0; k < V; ++k)
                if (x0 + k >= w) set_packed<NP>(r[i], k, 0u);
    }
    collide_store_packed<S, V, SR, (V / 2 >= 4) && LBM_ROLL_WRAP>(a, y, x0, r);
}

// One time step of one lattice.  Phase A issues every global load of the
// thread (3 mask rows, 9 population vectors and the warp-edge scalars) before
// any of them is consumed, so a thread has ~150 B in flight and pays one
// memory latency; phase B realigns the +-1 column shifts with shuffles and
// classifies boundary links; phase C fetches the cell's own opposite
// populations for bounce-back links (only near walls and solids); phase D
// collides and stores.
template <class S, int V, int FRAME, bool FAST, bool SR = false, bool EDGE = true, class A>
__device__ __forceinline__ void step_general(const A& a, int y,
                                             int tile, int lane) {
    using CT = typename Store<S>::CT;
    using ST = Store<S>;
    using IO = VecIO<S, V>;
    constexpr uint32_t FULL = (1u << V) - 1u;

    const int w = a.w, h = a.h;
    const int x0 = (tile * 32 + lane) * V;
    const bool active = x0 < w;
    const int xl = active ? x0 : 0;            // idle lanes read a valid chunk
    const S* __restrict__ src = static_cast<const S*>(a.src);
    const int64_t P = a.pitch, PL = a.plane;
    const int xm = a.flags & 3, ym = (a.flags >> 2) & 3;
    const bool halfway = (a.flags & LBM_SOLID_HALFWAY) != 0;
    const bool has_solid = a.solid != nullptr;
    const bool xper = xm == 1;
    const bool left_edge = lane == 0 || (EDGE && x0 == 0);          // needs column x0 - 1 itself
    const bool right_edge = lane == 31 || (EDGE && x0 + V >= w);    // needs column x0 + V itself

    // ---- phase A: issue all loads ----------------------------------------
    uint32_t mcore[3] = {0u, 0u, 0u}, mleft[3] = {0u, 0u, 0u}, mright[3] = {0u, 0u, 0u};
    if (has_solid) {
#pragma unroll
        for (int r = 0; r < 3; ++r) {
            int row = y - 1 + r;
            bool ok = true;
            if (EDGE && (row < 0 || row >= h)) {
                if (ym == 1) row = row < 0 ? row + h : row - h;
                else ok = false;
            }
            if (ok) {   // warp-uniform
                const uint8_t* mr = a.solid + int64_t(row) * a.mpitch;
                mcore[r] = load_mask_core<V>(mr + xl);
                if (left_edge) mleft[r] = EDGE ? mask_at(mr, x0 - 1, w, xper) : __ldg(mr + x0 - 1);
                if (right_edge) mright[r] = EDGE ? mask_at(mr, x0 + V, w, xper) : __ldg(mr + x0 + V);
            }
        }
    }

    S raw[9][V];
    S edge[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) {
        const int dc = DCOL(FRAME, i), dr = DROW(FRAME, i);
        int cls = 0;
        const int sr = EDGE ? source_row(y, dr, h, ym, &cls) : y - dr;
        const S* prow = src + i * PL + int64_t(sr) * P;
        IO::load(prow + xl, raw[i]);
        edge[i] = raw[i][0];
        if (dc == 1) {
            int ec = x0 - 1;
            if (EDGE && ec < 0) ec = xper ? w - 1 : -1;
            if (left_edge && ec >= 0) edge[i] = __ldg(prow + ec);
        } else if (dc == -1) {
            int ec = x0 + V;
            if (EDGE && ec >= w) ec = (xper && ec == w) ? 0 : -1;
            if (right_edge && ec >= 0) edge[i] = __ldg(prow + ec);
        }
    }

    // ---- phase B: realign, classify ---------------------------------------
    uint32_t mrow[3] = {0u, 0u, 0u};
    if (has_solid) {
#pragma unroll
        for (int r = 0; r < 3; ++r) {
            uint32_t core = mcore[r];
            const uint32_t l = __shfl_up_sync(kFull, (core >> (V - 1)) & 1u, 1);
            const uint32_t rr = __shfl_down_sync(kFull, core & 1u, 1);
            if (EDGE && x0 + V > w && xper) {    // partial last chunk, periodic: wrap
                int row = y - 1 + r;
                if (row < 0) row += h;
                if (row >= h) row -= h;
                const uint8_t* mr = a.solid + int64_t(row) * a.mpitch;
#pragma unroll
                for (int k = 0; k < V; ++k)
                    if (x0 + k >= w) core = (core & ~(1u << k)) | (mask_at(mr, x0 + k, w, true) << k);
            }
            mrow[r] = (left_edge ? mleft[r] : l) | (core << 1) | ((right_edge ? mright[r] : rr) << (V + 1));
        }
    }

    CT f[9][V];
    uint32_t bnc[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) {
        const int dc = DCOL(FRAME, i), dr = DROW(FRAME, i);
        const CT wi = a.c.wt[i];
        CT v[V];
        ST::dec_vec_dom(raw[i], v);
        const CT e = ST::dec_dom(edge[i]);
        uint32_t xz = 0u, xb = 0u;
        if (dc == 1) {
            const CT left = __shfl_up_sync(kFull, v[V - 1], 1);
#pragma unroll
            for (int k = V - 1; k > 0; --k) v[k] = v[k - 1];
            v[0] = left_edge ? e : left;
            if (EDGE && x0 == 0 && !xper) { if (xm == 2) xb |= 1u; else xz |= 1u; }
        } else if (dc == -1) {
            const CT right = __shfl_down_sync(kFull, v[0], 1);
#pragma unroll
            for (int k = 0; k < V - 1; ++k) v[k] = v[k + 1];
            v[V - 1] = right_edge ? e : right;
            if (EDGE && x0 + V >= w) {           // the row's last chunk (rare)
                int cls;
                const S* prow = src + i * PL + int64_t(source_row(y, dr, h, ym, &cls)) * P;
#pragma unroll
                for (int k = 0; k < V; ++k) {
                    const int sx = x0 + k + 1;
                    if (sx >= w) {
                        if (xper) {
                            if (!(k == V - 1 && sx == w))   // not already the edge load
                                v[k] = ST::dec_dom(__ldg(prow + (sx % w)));
                        } else if (xm == 2) {
                            xb |= 1u << k;
                        } else {
                            xz |= 1u << k;
                        }
                    }
                }
            }
        }
        int cls = 0;
        if (EDGE) (void)source_row(y, dr, h, ym, &cls);
        uint32_t b = (cls == 2) ? FULL : xb;
        const uint32_t z = (cls == 1 ? FULL : xz) & ~b;
        if (has_solid && halfway) b |= (mrow[1 - dr] >> (1 - dc)) & FULL;
        if (z) {
            const CT zv = ST::zero_dom(wi, a.c.dscale);
#pragma unroll
            for (int k = 0; k < V; ++k) if ((z >> k) & 1u) v[k] = zv;
        }
#pragma unroll
        for (int k = 0; k < V; ++k) f[i][k] = v[k];
        bnc[i] = b;
    }

    // ---- phase C: bounce-back links take the cell's own opposite population
#pragma unroll
    for (int i = 1; i < 9; ++i) {
        if (bnc[i]) {
            S own[V];
            IO::load(src + OPP(i) * PL + int64_t(y) * P + xl, own);
#pragma unroll
            for (int k = 0; k < V; ++k)
                if ((bnc[i] >> k) & 1u) f[i][k] = ST::dec_dom(own[k]);
        }
    }

    const uint32_t own_solid = has_solid ? ((mrow[1] >> 1) & FULL) : 0u;
    if (own_solid && !halfway) {
        // bounce_back (src/lbm.rs:741-751): solid nodes take swapped populations.
#pragma unroll
        for (int k = 0; k < V; ++k) {
            if ((own_solid >> k) & 1u) {
                CT t;
                t = f[1][k]; f[1][k] = f[3][k]; f[3][k] = t;
                t = f[2][k]; f[2][k] = f[4][k]; f[4][k] = t;
                t = f[5][k]; f[5][k] = f[7][k]; f[7][k] = t;
                t = f[6][k]; f[6][k] = f[8][k]; f[8][k] = t;
            }
        }
    }

    // ---- phase D: collide and write ---------------------------------------
    if (EDGE && SR && x0 + V > w) zero_past_edge<S, V>(f, x0, w);
    S enc[9][V];
    collide_cells<S, V, FAST>(a.c, f);
#pragma unroll
    for (int i = 0; i < 9; ++i) ST::enc_vec_dom(f[i], enc[i], SR ? 1 : 0);

    if (own_solid && halfway) {
        // Half-way mode: solid nodes keep their populations.
#pragma unroll
        for (int i = 0; i < 9; ++i) {
            S own[V];
            IO::load(src + i * PL + int64_t(y) * P + xl, own);
#pragma unroll
            for (int k = 0; k < V; ++k)
                if ((own_solid >> k) & 1u) enc[i][k] = own[k];
        }
    }

    if (!active) return;
    store_cells<S, V, FAST>(a, y, x0, enc);
}

// General tile of 16-bit storage, packed: the rules of step_general with the
// values kept two per register.  Bounce-back links, the solid swap and the
// half-way keep move raw 16-bit values (exact in either form); zero-padded
// links are substituted after widening, where the value f = 0 has its exact
// f32 deviation form.
template <class S, int V, int FRAME, bool SR, bool EDGE = true>
__device__ __forceinline__ void step_general_packed(const StepArgs<float>& a, int y, int tile,
                                                    int lane) {
    constexpr int NP = V / 2;
    constexpr uint32_t FULL = (1u << V) - 1u;
    const int w = a.w, h = a.h;
    const int x0 = (tile * 32 + lane) * V;
    const bool active = x0 < w;
    const int xl = active ? x0 : 0;
    const unsigned short* __restrict__ src = static_cast<const unsigned short*>(a.src);
    const int64_t P = a.pitch, PL = a.plane;
    const int xm = a.flags & 3, ym = (a.flags >> 2) & 3;
    const bool halfway = (a.flags & LBM_SOLID_HALFWAY) != 0;
    const bool has_solid = a.solid != nullptr;
    const bool xper = xm == 1;
    const bool left_edge = lane == 0 || (EDGE && x0 == 0);
    const bool right_edge = lane == 31 || (EDGE && x0 + V >= w);

    // ---- phase A: issue all loads ----------------------------------------
    uint32_t mcore[3] = {0u, 0u, 0u}, mleft[3] = {0u, 0u, 0u}, mright[3] = {0u, 0u, 0u};
    if (has_solid) {
#pragma unroll
        for (int r = 0; r < 3; ++r) {
            int row = y - 1 + r;
            bool ok = true;
            if (EDGE && (row < 0 || row >= h)) {
                if (ym == 1) row = row < 0 ? row + h : row - h;
                else ok = false;
            }
            if (ok) {
                const uint8_t* mr = a.solid + int64_t(row) * a.mpitch;
                mcore[r] = load_mask_core<V>(mr + xl);
                if (left_edge) mleft[r] = EDGE ? mask_at(mr, x0 - 1, w, xper) : __ldg(mr + x0 - 1);
                if (right_edge) mright[r] = EDGE ? mask_at(mr, x0 + V, w, xper) : __ldg(mr + x0 + V);
            }
        }
    }
    uint32_t r[9][NP];
    uint32_t edge[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) {
        const int dc = DCOL(FRAME, i), dr = DROW(FRAME, i);
        int cls = 0;
        const int sr = EDGE ? source_row(y, dr, h, ym, &cls) : y - dr;
        const unsigned short* prow = src + i * PL + int64_t(sr) * P;
        PackIO<NP>::load(prow + xl, r[i]);
        edge[i] = 0u;
        if (dc == 1) {
            int ec = x0 - 1;
            if (EDGE && ec < 0) ec = xper ? w - 1 : -1;
            if (left_edge && ec >= 0) edge[i] = uint32_t(__ldg(prow + ec)) << 16;
        } else if (dc == -1) {
            int ec = x0 + V;
            if (EDGE && ec >= w) ec = (xper && ec == w) ? 0 : -1;
            if (right_edge && ec >= 0) edge[i] = __ldg(prow + ec);
        }
    }

    // ---- phase B: realign, classify ---------------------------------------
    uint32_t mrow[3] = {0u, 0u, 0u};
    if (has_solid) {
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            uint32_t core = mcore[q];
            const uint32_t l = __shfl_up_sync(kFull, (core >> (V - 1)) & 1u, 1);
            const uint32_t rr = __shfl_down_sync(kFull, core & 1u, 1);
            if (EDGE && x0 + V > w && xper) {
                int row = y - 1 + q;
                if (row < 0) row += h;
                if (row >= h) row -= h;
                const uint8_t* mr = a.solid + int64_t(row) * a.mpitch;
#pragma unroll
                for (int k = 0; k < V; ++k)
                    if (x0 + k >= w) core = (core & ~(1u << k)) | (mask_at(mr, x0 + k, w, true) << k);
            }
            mrow[q] = (left_edge ? mleft[q] : l) | (core << 1) | ((right_edge ? mright[q] : rr) << (V + 1));
        }
    }
    uint32_t zb[9], bnc[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) {
        const int dc = DCOL(FRAME, i), dr = DROW(FRAME, i);
        uint32_t xz = 0u, xb = 0u;
        if (dc == 1) {
            const uint32_t left = __shfl_up_sync(kFull, r[i][NP - 1], 1);
            shift_up_packed<NP>(r[i], left_edge ? edge[i] : left);
            if (EDGE && x0 == 0 && !xper) { if (xm == 2) xb |= 1u; else xz |= 1u; }
        } else if (dc == -1) {
            const uint32_t right = __shfl_down_sync(kFull, r[i][0], 1);
            shift_down_packed<NP>(r[i], right_edge ? edge[i] : right);
            if (EDGE && x0 + V >= w) {           // the row's last chunk (rare)
                int cls;
                const unsigned short* prow = src + i * PL + int64_t(source_row(y, dr, h, ym, &cls)) * P;
#pragma unroll
                for (int k = 0; k < V; ++k) {
                    const int sx = x0 + k + 1;
                    if (sx >= w) {
                        if (xper) {
                            if (!(k == V - 1 && sx == w))
                                set_packed<NP>(r[i], k, __ldg(prow + (sx % w)));
                        } else if (xm == 2) {
                            xb |= 1u << k;
                        } else {
                            xz |= 1u << k;
                        }
                    }
                }
            }
        }
        int cls = 0;
        if (EDGE) (void)source_row(y, dr, h, ym, &cls);
        uint32_t b = (cls == 2) ? FULL : xb;
        const uint32_t z = (cls == 1 ? FULL : xz) & ~b;
        if (has_solid && halfway) b |= (mrow[1 - dr] >> (1 - dc)) & FULL;
        zb[i] = z & ~b;                          // a bounce-back link overrides padding
        bnc[i] = b;
    }

    // ---- phase C: bounce-back links take the cell's own opposite population
#pragma unroll
    for (int i = 1; i < 9; ++i) {
        if (bnc[i]) {
            uint32_t own[NP];
            PackIO<NP>::load(src + OPP(i) * PL + int64_t(y) * P + xl, own);
#pragma unroll
            for (int j = 0; j < NP; ++j) {
                const uint32_t m = half_mask(bnc[i], j);
                r[i][j] = (r[i][j] & ~m) | (own[j] & m);
            }
        }
    }
    const uint32_t own_solid = has_solid ? ((mrow[1] >> 1) & FULL) : 0u;
    if (own_solid && !halfway) {
        // bounce_back (src/lbm.rs:741-751): solid nodes take swapped
        // populations; a zero-padded link moves with its value (w_i equals
        // w_opp(i), so the substitute is the same)
#pragma unroll
        for (int p = 0; p < 4; ++p) {
            const int i0 = p < 2 ? 1 + p : 5 + (p - 2), i1 = OPP(i0);
#pragma unroll
            for (int j = 0; j < NP; ++j) {
                const uint32_t m = half_mask(own_solid, j);
                const uint32_t t = (r[i0][j] ^ r[i1][j]) & m;
                r[i0][j] ^= t;
                r[i1][j] ^= t;
            }
            const uint32_t t = (zb[i0] ^ zb[i1]) & own_solid;
            zb[i0] ^= t;
            zb[i1] ^= t;
        }
    }

    // ---- phase D: collide and write ---------------------------------------
    const uint32_t past = (EDGE && x0 + V > w) ? (FULL << (w - x0 > 0 ? w - x0 : 0)) & FULL : 0u;
    collide_packed<S, V, SR, true, (V / 2 >= 4)>(a.c, r, zb, past);
    if (own_solid && halfway) {
        // half-way mode: solid nodes keep their populations
#pragma unroll
        for (int i = 0; i < 9; ++i) {
            uint32_t own[NP];
            PackIO<NP>::load(src + i * PL + int64_t(y) * P + xl, own);
#pragma unroll
            for (int j = 0; j < NP; ++j) {
                const uint32_t m = half_mask(own_solid, j);
                r[i][j] = (r[i][j] & ~m) | (own[j] & m);
            }
        }
    }
    if (!active) return;
    store_packed<S, V>(a, y, x0, r);
}

// A listed (general) tile.
template <class S, int V, int FRAME, bool FAST, bool SR, bool EDGE>
__device__ __forceinline__ void step_listed(const StepArgs<typename Store<S>::CT>& a, int y, int tile) {
    if constexpr (Store<S>::DEV && LBM_PACKED16) step_general_packed<S, V, FRAME, SR, EDGE>(a, y, tile, threadIdx.x);
    else step_general<S, V, FRAME, FAST, SR, EDGE>(a, y, tile, threadIdx.x);
}

// One step over the whole lattice in one launch.  With tile flags: the first
// ceil(ngtiles / rows) blocks take the listed tiles from a.gtiles (entry =
// row * ntiles + tile, bit 31 set for flag 3), one warp per entry, so their
// longer latency overlaps the rest; the remaining blocks cover every (row,
// tile) in row-major order and run the interior paths, leaving tiles flagged
// 1 or 3 to the list.  Without tile flags, every tile takes the general path.
// Resident blocks of 256 threads the register allocation is sized for: 3 at
// 4 cells per thread (f32 and 16-bit), 2 for 16-bit at 8 cells, 1 otherwise.
#ifndef LBM_STEP_MIN_BLOCKS
#define LBM_STEP_MIN_BLOCKS 3
#endif
#ifndef LBM_STEP_MIN_BLOCKS_16
#define LBM_STEP_MIN_BLOCKS_16 3
#endif
#ifndef LBM_STEP_MIN_BLOCKS_16_V8
#define LBM_STEP_MIN_BLOCKS_16_V8 2
#endif
template <class S, int V>
constexpr int step_min_blocks() {
    if (sizeof(typename Store<S>::CT) != 4) return 1;
    if (sizeof(S) == 2) return V <= 4 ? LBM_STEP_MIN_BLOCKS_16 : LBM_STEP_MIN_BLOCKS_16_V8;
    return V <= 4 ? LBM_STEP_MIN_BLOCKS : 1;
}
template <class S, int V, int FRAME, bool FAST, bool SR>
__device__ __forceinline__ void step_block(const StepArgs<typename Store<S>::CT>& a) {
    const int rows = blockDim.y;
    const int gblocks = a.tflags != nullptr ? (a.ngtiles + rows - 1) / rows : 0;
    const int b = blockIdx.x;
    if (b < gblocks) {
        const int e = b * rows + threadIdx.y;
        if (e >= a.ngtiles) return;
        const uint32_t entry = a.gtiles[e];
        const uint32_t t = entry & 0x7fffffffu;
        const int y = int(t / uint32_t(a.ntiles));
        const int tile = int(t - uint32_t(y) * uint32_t(a.ntiles));
        if (entry >> 31) {       // solids nearby, no lattice edge within reach (warp-uniform)
            step_listed<S, V, FRAME, FAST, SR, false>(a, y, tile);
        } else {
            step_listed<S, V, FRAME, FAST, SR, true>(a, y, tile);
        }
        return;
    }
    const int ib = b - gblocks;
    const int by = ib / a.ntiles, tile = ib - by * a.ntiles;
    const int y = by * rows + threadIdx.y;
    if (y >= a.h) return;                                                  // warp-uniform
    if (a.tflags == nullptr) {
        step_listed<S, V, FRAME, FAST, SR, true>(a, y, tile);
        return;
    }
    const uint8_t flag = a.tflags[int64_t(y) * a.ntiles + tile];        // warp-uniform
    const int x0 = (tile * 32 + threadIdx.x) * V;
    if constexpr (Store<S>::DEV && LBM_PACKED16) {
        // 1 and 3 are owned by the list, except 3 when link masks exist
        if (flag == 1 || (flag == 3 && a.links == nullptr)) return;
        if (flag == 2) step_interior_wrap_packed<S, V, FRAME, SR>(a, y, x0, threadIdx.x);
        else if (flag == 3) step_interior_packed<S, V, FRAME, SR, true>(a, y, x0, threadIdx.x, tile);
        else step_interior_packed<S, V, FRAME, SR>(a, y, x0, threadIdx.x);
    } else {
        // 1 and 3 are owned by the list, except 3 when link masks exist
        if (flag == 1 || (flag == 3 && a.links == nullptr)) return;
        if (flag == 0) step_interior<S, V, FRAME, FAST, SR>(a, y, x0, threadIdx.x);
        else if (flag == 3) {
            if constexpr (LBM_LINKS_F32 && std::is_same<S, float>::value)
                step_interior<S, V, FRAME, FAST, SR, true>(a, y, x0, threadIdx.x, tile);
        }
        else step_interior_wrap<S, V, FRAME, FAST, SR>(a, y, x0, threadIdx.x);
    }
}

// The step kernels.  16-bit storage at 8 cells per thread is capped at 96
// registers (5 blocks of 4 warps per SM, ~300 B of spills in the general
// paths) instead of 128 (4 blocks): 4096^2 obstacle channel, stochastic
// rounding, one GB300: 156.4k -> 160.2k MLUPS (88 registers 156.2k, 104
// registers 149.8k).  Every other kernel is sized by step_min_blocks.
#ifndef LBM_STEP16_V8_MAXNREG
#define LBM_STEP16_V8_MAXNREG 96
#endif
template <class S, int V, int FRAME, bool FAST, bool SR>
__global__ void __launch_bounds__(256, step_min_blocks<S, V>())
lbm_step_kernel(const StepArgs<typename Store<S>::CT> a) {
    step_block<S, V, FRAME, FAST, SR>(a);
}
template <class S, int V, int FRAME, bool FAST, bool SR>
__global__ void __maxnreg__(LBM_STEP16_V8_MAXNREG)
lbm_step_kernel_capped(const StepArgs<typename Store<S>::CT> a) {
    step_block<S, V, FRAME, FAST, SR>(a);
}

template <class S, int V>
constexpr bool step_capped() { return sizeof(S) == 2 && V == 8; }

// Prefetch distance, in percent of the rows the resident blocks cover (the
// wavefront's depth): far enough that the prefetched rows arrive before
// their warps start, near enough that they are still in L2.
#ifndef LBM_PREFETCH_PCT
#define LBM_PREFETCH_PCT 60
#endif

template <class S, int V, int FRAME, bool FAST, bool SR>
void launch_step_tv(const StepArgs<typename Store<S>::CT>& a, int rows, cudaStream_t stream) {
    const int ntiles = (a.w + 32 * V - 1) / (32 * V);
    const int rowblocks = (a.h + rows - 1) / rows;
    const int gblocks = a.tflags != nullptr ? (a.ngtiles + rows - 1) / rows : 0;
    StepArgs<typename Store<S>::CT> b = a;
    b.ntiles = ntiles;
    if (b.pf_rows < 0) {
        // Resident blocks per SM of this kernel at each block size, times
        // the SMs: computed once per instantiation (thread-safe static
        // initialisation; one GPU model per process).  0 turns the prefetch off.
        static const std::array<int, 9> blocks_per_gpu = [] {
            std::array<int, 9> out{};
            int dev = 0, sms = 0;
            if (cudaGetDevice(&dev) != cudaSuccess ||
                cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
                return out;
            for (int r = 1; r <= 8; ++r) {
                int occ = 0;
                cudaError_t e;
                if constexpr (step_capped<S, V>())
                    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                        &occ, lbm_step_kernel_capped<S, V, FRAME, FAST, SR>, 32 * r, 0);
                else
                    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                        &occ, lbm_step_kernel<S, V, FRAME, FAST, SR>, 32 * r, 0);
                if (e == cudaSuccess) out[r] = occ * sms;
            }
            (void)cudaGetLastError();
            return out;
        }();
        const int64_t wave_rows = int64_t(blocks_per_gpu[rows]) * rows / ntiles;
        b.pf_rows = int(wave_rows * LBM_PREFETCH_PCT / 100);
    }
    const int grid = gblocks + ntiles * rowblocks;
    if constexpr (step_capped<S, V>())
        lbm_step_kernel_capped<S, V, FRAME, FAST, SR><<<grid, dim3(32, rows), 0, stream>>>(b);
    else
        lbm_step_kernel<S, V, FRAME, FAST, SR><<<grid, dim3(32, rows), 0, stream>>>(b);
}

// One step: the interior kernel plus the general kernel over the flagged
// tiles (with tile flags), or the general kernel over every tile (without).
template <class S, int V>
cudaError_t launch_step_v(const StepArgs<typename Store<S>::CT>& a, int frame, bool fast,
                          int rows, cudaStream_t stream) {
    (void)cudaGetLastError();   // report this launch's status, not an earlier call's
    // 16-bit storage: the rounding of the stores is a compile-time choice
    // (a runtime choice between the two conversions cost about 4%)
    if constexpr (Store<S>::DEV) {
        if (a.c.stochastic) {
            if (frame) {
                if (fast) launch_step_tv<S, V, 1, true, true>(a, rows, stream);
                else launch_step_tv<S, V, 1, false, true>(a, rows, stream);
            } else {
                if (fast) launch_step_tv<S, V, 0, true, true>(a, rows, stream);
                else launch_step_tv<S, V, 0, false, true>(a, rows, stream);
            }
            return cudaGetLastError();
        }
    }
    if (frame) {
        if (fast) launch_step_tv<S, V, 1, true, false>(a, rows, stream);
        else launch_step_tv<S, V, 1, false, false>(a, rows, stream);
    } else {
        if (fast) launch_step_tv<S, V, 0, true, false>(a, rows, stream);
        else launch_step_tv<S, V, 0, false, false>(a, rows, stream);
    }
    return cudaGetLastError();
}

}  // namespace lbmk
