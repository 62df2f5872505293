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
template <> struct Store<float> {
    using CT = float;
    static constexpr bool DEV = false;
    __device__ static float dec(float s, float, float) { return s; }
    __device__ static float enc(float f, float, float) { return f; }
};
template <> struct Store<double> {
    using CT = double;
    static constexpr bool DEV = false;
    __device__ static double dec(double s, double, double) { return s; }
    __device__ static double enc(double f, double, double) { return f; }
};
template <> struct Store<__half> {
    using CT = float;
    static constexpr bool DEV = true;
    __device__ static float dec(__half s, float w, float inv_scale) {
        return __fmaf_rn(__half2float(s), inv_scale, w);
    }
    __device__ static __half enc(float f, float w, float scale) {
        return __float2half_rn(__fmul_rn(__fsub_rn(f, w), scale));
    }
};
template <> struct Store<__nv_bfloat16> {
    using CT = float;
    static constexpr bool DEV = true;
    __device__ static float dec(__nv_bfloat16 s, float w, float inv_scale) {
        return __fmaf_rn(__bfloat162float(s), inv_scale, w);
    }
    __device__ static __nv_bfloat16 enc(float f, float w, float scale) {
        return __float2bfloat16_rn(__fmul_rn(__fsub_rn(f, w), scale));
    }
};

// Power-of-two scale of the deviation formats: keeps |f_i - w_i| >= 1e-8
// out of the half subnormal range while |f_i - w_i| <= 7 still fits.
constexpr float kHalfDevScale = 8192.0f;
constexpr float kBf16DevScale = 1.0f;

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
    int collision;          // LBM_COLLISION_*
    int force;              // nonzero when a body force is set
};

// Arguments of one fused step over one lattice.
template <class CT>
struct StepArgs {
    const void* src;        // 9 planes, current state
    void* dst;              // 9 planes, next state
    const uint8_t* solid;   // mask (pitch mpitch) or null
    float* mom_rho;         // moment outputs (pitch `pitch`) or null
    float* mom_ux;
    float* mom_uy;
    int w, h, pitch, mpitch;
    int64_t plane;          // plane stride in elements
    int flags;
    Consts<CT> c;
};

// Strict arithmetic: one IEEE rounding per operation, no contraction; the
// operation order of src/lbm.rs.  Fast arithmetic: contracted / simplified.
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
    __device__ static float rcp(float a) { return __frcp_rn(a); }
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
