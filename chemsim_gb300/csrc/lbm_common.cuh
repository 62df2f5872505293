// lbm_common.cuh — shared definitions of the sm_103a D2Q9 kernels.
//
// Direction order, weights and velocities are those of D2Q9::directions
// (taktoa/chemsim src/lbm.rs:202-282); the opposite map is swap_populations
// (src/lbm.rs:298-309).
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/lbm_cuda.h"

namespace lbmk {

// c_i = (cx, cy), src/lbm.rs:217-227.
__host__ __device__ constexpr int CX(int i) {
    return (i == 1 || i == 5 || i == 8) ? 1 : ((i == 3 || i == 6 || i == 7) ? -1 : 0);
}
__host__ __device__ constexpr int CY(int i) {
    return (i == 2 || i == 5 || i == 6) ? 1 : ((i == 4 || i == 7 || i == 8) ? -1 : 0);
}
// swap_populations: 1<->3, 2<->4, 5<->7, 6<->8.
__host__ __device__ constexpr int OPP(int i) {
    return i == 0 ? 0 : (i <= 4 ? ((i + 1) % 4) + 1 : ((i - 3) % 4) + 5);
}
// Grid displacement of direction i (column, row).  Frame 0 (REF): the
// convolve2 of src/lbm.rs:716-729 moves plane i by (drow, dcol) = (-cx, +cy);
// frame 1 (XY): (dcol, drow) = (+cx, +cy).
__host__ __device__ constexpr int DCOL(int frame, int i) { return frame ? CX(i) : CY(i); }
__host__ __device__ constexpr int DROW(int frame, int i) { return frame ? CY(i) : -CX(i); }

static_assert(OPP(1) == 3 && OPP(2) == 4 && OPP(3) == 1 && OPP(4) == 2, "opp");
static_assert(OPP(5) == 7 && OPP(6) == 8 && OPP(7) == 5 && OPP(8) == 6, "opp");

// Storage traits: S is the stored element type, CT the collision type.
// Deviation storage keeps (f_i - w_i) * scale in 16 bits.
template <class S> struct Store;
// Plain storage: decode / encode are the identity.
template <class T>
struct PlainStore {
    using CT = T;
    static constexpr bool DEV = false;
    __device__ static T dec(T s, T, T) { return s; }
    __device__ static T enc(T f, T, T) { return f; }
    template <int V>
    __device__ static void dec_vec(const T (&s)[V], T (&f)[V], T, T) {
#pragma unroll
        for (int k = 0; k < V; ++k) f[k] = s[k];
    }
    template <int V>
    __device__ static void enc_vec(const T (&f)[V], T (&s)[V], T, T) {
#pragma unroll
        for (int k = 0; k < V; ++k) s[k] = f[k];
    }
    // The step kernels' working variables ("domain"): f itself.
    __device__ static T dec_dom(T s) { return s; }
    __device__ static T zero_dom(T, T) { return T(0); }
    template <int V>
    __device__ static void dec_vec_dom(const T (&s)[V], T (&f)[V]) {
#pragma unroll
        for (int k = 0; k < V; ++k) f[k] = s[k];
    }
    template <int V>
    __device__ static void enc_vec_dom(const T (&f)[V], T (&s)[V], int) {
#pragma unroll
        for (int k = 0; k < V; ++k) s[k] = f[k];
    }
};
template <> struct Store<float> : PlainStore<float> {};
template <> struct Store<double> : PlainStore<double> {};
// 16-bit deviation storage; the vector forms convert element pairs with one
// paired conversion instruction.
template <class H, class H2>
struct DevStore {
    using CT = float;
    static constexpr bool DEV = true;
    __device__ static float to_f(H s);
    __device__ static H from_f(float f);
    __device__ static float2 to_f2(H2 s);
    __device__ static H2 from_f2(float2 f);
    __device__ static float dec(H s, float w, float inv_scale) {
        return __fmaf_rn(to_f(s), inv_scale, w);
    }
    __device__ static H enc(float f, float w, float scale) {
        return from_f(__fmul_rn(__fsub_rn(f, w), scale));
    }
    template <int V>
    __device__ static void dec_vec(const H (&s)[V], float (&f)[V], float w, float inv_scale) {
        static_assert(V % 2 == 0, "pairs");
#pragma unroll
        for (int k = 0; k < V; k += 2) {
            H2 p;
            memcpy(&p, &s[k], sizeof(H2));
            const float2 q = to_f2(p);
            f[k] = __fmaf_rn(q.x, inv_scale, w);
            f[k + 1] = __fmaf_rn(q.y, inv_scale, w);
        }
    }
    template <int V>
    __device__ static void enc_vec(const float (&f)[V], H (&s)[V], float w, float scale) {
        static_assert(V % 2 == 0, "pairs");
#pragma unroll
        for (int k = 0; k < V; k += 2) {
            const H2 p = from_f2(make_float2(__fmul_rn(__fsub_rn(f[k], w), scale),
                                             __fmul_rn(__fsub_rn(f[k + 1], w), scale)));
            memcpy(&s[k], &p, sizeof(H2));
        }
    }
    // The step kernels' working variables ("domain"): the scaled deviation
    // G_i = s (f_i - w_i) itself, so loading and storing are bare conversions.
    __device__ static float dec_dom(H s) { return to_f(s); }
    __device__ static float zero_dom(float w, float scale) { return -w * scale; }   // f = 0
    template <int V>
    __device__ static void dec_vec_dom(const H (&s)[V], float (&f)[V]) {
#pragma unroll
        for (int k = 0; k < V; k += 2) {
            H2 p;
            memcpy(&p, &s[k], sizeof(H2));
            const float2 q = to_f2(p);
            f[k] = q.x;
            f[k + 1] = q.y;
        }
    }
    // Stores the collided values.  With `stochastic` each value is rounded
    // stochastically (the hardware conversion, random bits hashed from the
    // values' own f32 bits, so the result is reproducible).  Rounding to
    // nearest repeats the same error on a slowly changing field step after
    // step, and those errors add up; stochastic rounding averages them out
    // (the u error of a laminar 1024^2 Taylor-Green run after 5000 steps
    // drops from 1.6e-2 to 7e-4 against f64).
    template <int V>
    __device__ static void enc_vec_dom(const float (&f)[V], H (&s)[V], int stochastic) {
#pragma unroll
        for (int k = 0; k < V; k += 2) {
            const H2 p = stochastic ? from_f2_sr(f[k], f[k + 1]) : from_f2(make_float2(f[k], f[k + 1]));
            memcpy(&s[k], &p, sizeof(H2));
        }
    }
    __device__ static H2 from_f2_sr(float lo, float hi);
};

template <> __device__ inline float DevStore<__half, __half2>::to_f(__half s) { return __half2float(s); }
template <> __device__ inline __half DevStore<__half, __half2>::from_f(float f) { return __float2half_rn(f); }
template <> __device__ inline float2 DevStore<__half, __half2>::to_f2(__half2 s) { return __half22float2(s); }
template <> __device__ inline __half2 DevStore<__half, __half2>::from_f2(float2 f) { return __float22half2_rn(f); }
template <> __device__ inline float DevStore<__nv_bfloat16, __nv_bfloat162>::to_f(__nv_bfloat16 s) { return __bfloat162float(s); }
template <> __device__ inline __nv_bfloat16 DevStore<__nv_bfloat16, __nv_bfloat162>::from_f(float f) { return __float2bfloat16_rn(f); }
template <> __device__ inline float2 DevStore<__nv_bfloat16, __nv_bfloat162>::to_f2(__nv_bfloat162 s) { return __bfloat1622float2(s); }
template <> __device__ inline __nv_bfloat162 DevStore<__nv_bfloat16, __nv_bfloat162>::from_f2(float2 f) { return __float22bfloat162_rn(f); }
// Random bits of a pair for the stochastic-rounding conversion: one
// multiply-add of both values' f32 bits (the low bits that a conversion
// drops are noise-like, and the multiply spreads each value's bits upward),
// so a run is reproducible bit for bit.  Two multiplies and an xor measured
// no more accurate and 3-4% slower.
__device__ __forceinline__ uint32_t sr_bits(float lo, float hi) {
    return __float_as_uint(lo) * 0x9E3779B1u + __float_as_uint(hi);
}
// cvt.rs: the hardware stochastic-rounding conversion of sm_100-class GPUs.
template <>
__device__ inline __half2 DevStore<__half, __half2>::from_f2_sr(float lo, float hi) {
    uint32_t d;
    asm("cvt.rs.f16x2.f32 %0, %1, %2, %3;" : "=r"(d) : "f"(hi), "f"(lo), "r"(sr_bits(lo, hi)));
    __half2 out;
    memcpy(&out, &d, 4);
    return out;
}
template <>
__device__ inline __nv_bfloat162 DevStore<__nv_bfloat16, __nv_bfloat162>::from_f2_sr(float lo, float hi) {
    uint32_t d;
    asm("cvt.rs.bf16x2.f32 %0, %1, %2, %3;" : "=r"(d) : "f"(hi), "f"(lo), "r"(sr_bits(lo, hi)));
    __nv_bfloat162 out;
    memcpy(&out, &d, 4);
    return out;
}
template <> struct Store<__half> : DevStore<__half, __half2> {};
template <> struct Store<__nv_bfloat16> : DevStore<__nv_bfloat16, __nv_bfloat162> {};

// Power-of-two scale of the deviation formats: keeps |f_i - w_i| >= 1e-8
// out of the half subnormal range while |f_i - w_i| <= 7 still fits.
constexpr float kHalfDevScale = 8192.0f;
constexpr float kBf16DevScale = 1.0f;

// Constants of the folded BGK collision of deviation variables on cell pairs
// (collide_bgk_folded_x2), each value stored in both halves of a float2 so
// that the packed f32x2 instructions read it as one 64-bit operand.  With
// omega = dt/tau and the weight classes c = rest (w_0), axis (w_1 = w_2 = w_3
// = w_4) and diagonal (w_5 = ... = w_8), omega G_eq_i + S_i (Guo) is
//   [omega w_c D - sgw_c uF + a_c E_i + sgw_i cF4_i (c_i.u)] +- [a_c k1 (c_i.u) + sgw_i kcF_i]
// (D = sum G, a_c = omega w_c s rho, E_i = k2 (c_i.u)^2 + k3 u^2, uF = k1 u.F):
// the first bracket is even and the second odd under c_i -> -c_i, so a
// direction pair (i, opp(i)) shares both, and out_i = keep G_i + that.
struct PairConsts {
    float2 keep;        // 1 - dt/tau
    float2 ow[3];       // omega w_c
    float2 owk[3];      // omega w_c k1
    float2 k2, k3;
    float2 k1fx, k1fy;  // k1 F: uF = ux k1fx + uy k1fy
    float2 nsgw[3];     // -(s guo w_c)
    float2 sgwcF4[9];   // s guo w_i cF4_i
    float2 so[9];       // s guo w_i kcF_i
    float2 dscale, shfx, shfy;
};

// Collision constants, computed on the host in the collision type exactly as
// src/lbm.rs computes them (see lbm_api.cu: make_consts).
template <class CT>
struct Consts {
    CT wt[9];
    CT k1, k2, k3;          // 1/cs2, 1/(2 cs4), -1/(2 cs2)
    CT bgk_factor;          // -dt/tau
    CT omega_p, omega_m;    // TRT 1/tau_plus, 1/tau_minus
    CT trt_scale;           // -dt*0.5
    CT fx, fy, hfx, hfy;    // body force and half of it
    CT guo;                 // 1 - 1/(2 tau)
    CT inv_cs4;
    CT dscale, dinv;        // deviation-storage scale and its inverse
    CT gw[9];               // guo * w_i                      (fast path)
    CT kcF[9];              // k1 * (c_i . F)                 (fast path)
    CT cF4[9];              // (c_i . F) / cs^4               (fast path)
    CT sgw[9];              // dscale * guo * w_i             (deviation form)
    CT shfx, shfy;          // dscale * F / 2                 (deviation form)
    int collision;          // LBM_COLLISION_*
    int stochastic;         // 16-bit storage: stochastic rounding (not LBM_ROUND_NEAREST)
    int force;              // nonzero when a body force is set
    PairConsts pk;          // the folded pair collision's constants (deviation storage)
};

// Fills c.pk from the scalar constants (host side, in double, rounded once).
template <class CT>
inline void fill_pair_consts(Consts<CT>& c) {
    auto b = [](double v) { return make_float2(float(v), float(v)); };
    const double om = -double(c.bgk_factor);
    const double dev = double(c.dscale);
    PairConsts& k = c.pk;
    k.keep = b(1.0 + double(c.bgk_factor));
    const int cls[3] = {0, 1, 5};
    for (int q = 0; q < 3; ++q) {
        const double wc = double(c.wt[cls[q]]);
        k.ow[q] = b(om * wc);
        k.owk[q] = b(om * wc * double(c.k1));
        k.nsgw[q] = b(-dev * double(c.gw[cls[q]]));
    }
    k.k2 = b(double(c.k2));
    k.k3 = b(double(c.k3));
    k.k1fx = b(double(c.k1) * double(c.fx));
    k.k1fy = b(double(c.k1) * double(c.fy));
    for (int i = 0; i < 9; ++i) {
        k.sgwcF4[i] = b(dev * double(c.gw[i]) * double(c.cF4[i]));
        k.so[i] = b(dev * double(c.gw[i]) * double(c.kcF[i]));
    }
    k.dscale = b(dev);
    k.shfx = b(double(c.shfx));
    k.shfy = b(double(c.shfy));
}

// Arguments of one fused step over one lattice.
// 1 (the default): f32 lattices with solids get per-lane link masks too, and
// their tiles flagged 3 take the interior path (step_interior with GEN_CT).
// 4096^2 obstacle channel, f32 fast, one GB300: 0.97 -> 1.015 of the copy
// bandwidth.
#ifndef LBM_LINKS_F32
#define LBM_LINKS_F32 1
#endif

template <class CT>
struct StepArgs {
    const void* src;        // 9 planes, current state
    void* dst;              // 9 planes, next state
    const uint8_t* solid;   // mask (pitch mpitch) or null
    const uint8_t* tflags;  // per (row, warp tile): 0 interior, 2 periodic edge, 1 / 3 listed, or null
    int ntiles;             // warp tiles per row (row stride of tflags)
    const uint32_t* gtiles; // listed tiles (row * ntiles + tile, bit 31: no lattice edge in reach), or null
    int ngtiles;
    const uint4* links;     // 16-bit storage at 8 cells per thread: per (tile, lane) link masks of
                            // the tiles flagged 3, which then take the interior path (or null)
    float* mom_rho;         // moment outputs (pitch `pitch`) or null
    float* mom_ux;
    float* mom_uy;
    int mom_pitch;          // row stride of the moment outputs in elements
    int w, h, pitch, mpitch;
    int64_t plane;          // plane stride in elements
    int flags;
    int pf_rows;            // L2 prefetch distance in rows: 0 off, < 0 chosen at launch
    Consts<CT> c;
};

// Strict arithmetic: one IEEE rounding per operation, no contraction; the
// operation order of src/lbm.rs.  Fast arithmetic: contracted / simplified.
#ifndef LBM_RCP_APPROX
#define LBM_RCP_APPROX 1
#endif
template <bool FAST> struct Ar;
template <> struct Ar<false> {
    __device__ static float add(float a, float b) { return __fadd_rn(a, b); }
    __device__ static float sub(float a, float b) { return __fsub_rn(a, b); }
    __device__ static float mul(float a, float b) { return __fmul_rn(a, b); }
    __device__ static float rcp(float a) { return __fdiv_rn(1.0f, a); }
    __device__ static double add(double a, double b) { return __dadd_rn(a, b); }
    __device__ static double sub(double a, double b) { return __dsub_rn(a, b); }
    __device__ static double mul(double a, double b) { return __dmul_rn(a, b); }
    __device__ static double rcp(double a) { return __ddiv_rn(1.0, a); }
};
template <> struct Ar<true> {
    __device__ static float add(float a, float b) { return a + b; }
    __device__ static float sub(float a, float b) { return a - b; }
    __device__ static float mul(float a, float b) { return a * b; }
#if LBM_RCP_APPROX
    // one MUFU reciprocal (max error about 1 ulp); densities never come near
    // the flush-to-zero range
    __device__ static float rcp(float a) {
        float r;
        asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(a));
        return r;
    }
#else
    __device__ static float rcp(float a) { return __frcp_rn(a); }
#endif
    __device__ static double add(double a, double b) { return a + b; }
    __device__ static double sub(double a, double b) { return a - b; }
    __device__ static double mul(double a, double b) { return a * b; }
    __device__ static double rcp(double a) { return 1.0 / a; }
};

// Launch of the fused step for one storage type (defined per type in
// lbm_step_<type>.cu).  cells_per_thread / rows_per_block select the tile.
template <class S>
cudaError_t launch_step(const StepArgs<typename Store<S>::CT>& a, int frame,
                        bool fast, int cells_per_thread, int rows_per_block,
                        cudaStream_t stream);

}  // namespace lbmk
