// lbm_aux.cuh — the non-hot kernels around the fused step: initial
// equilibrium, host-layout <-> device-layout conversion, moment readback and
// the f64 health reduction.  All use the reference's operation order (strict
// arithmetic) so their results match the oracle bit for bit in f32/f64.
#pragma once

#include <math.h>

#include <string>

#include "lbm_step.cuh"

namespace lbmk {

// compute_equilibrium of one cell (src/lbm.rs:43-71), strict order.
template <class CT>
__device__ __forceinline__ void equilibrium_strict(const Consts<CT>& c, CT rho, CT ux, CT uy,
                                                   CT (&feq)[9]) {
    using A = Ar<false>;
    const CT v2k3 = A::mul(A::add(A::mul(ux, ux), A::mul(uy, uy)), c.k3);
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
#pragma unroll
    for (int i = 0; i < 9; ++i) {
        CT s = A::add(CT(1), A::mul(vc[i], c.k1));
        s = A::add(s, A::mul(A::mul(vc[i], vc[i]), c.k2));
        s = A::add(s, v2k3);
        feq[i] = A::mul(A::mul(rho, c.wt[i]), s);
    }
}

// Populations <- f_eq(rho, u) from pitched f32 fields.
template <class S>
__global__ void eq_init_kernel(S* __restrict__ dst, const float* __restrict__ rho,
                               const float* __restrict__ ux, const float* __restrict__ uy,
                               int w, int h, int pitch, int64_t plane,
                               Consts<typename Store<S>::CT> c) {
    using CT = typename Store<S>::CT;
    const int64_t n = int64_t(w) * h;
    for (int64_t t = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; t < n;
         t += int64_t(gridDim.x) * blockDim.x) {
        const int y = int(t / w), x = int(t - int64_t(y) * w);
        const int64_t o = int64_t(y) * pitch + x;
        CT feq[9];
        equilibrium_strict<CT>(c, CT(rho[o]), CT(ux[o]), CT(uy[o]), feq);
#pragma unroll
        for (int i = 0; i < 9; ++i) dst[i * plane + o] = Store<S>::enc(feq[i], c.wt[i], c.dscale);
    }
}

// Rest state f_i = w_i in every cell (and padding column) of every plane.
template <class S>
__global__ void fill_rest_kernel(S* __restrict__ dst, int64_t plane,
                                 Consts<typename Store<S>::CT> c) {
    for (int64_t t = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; t < plane;
         t += int64_t(gridDim.x) * blockDim.x) {
#pragma unroll
        for (int i = 0; i < 9; ++i) dst[i * plane + t] = Store<S>::enc(c.wt[i], c.wt[i], c.dscale);
    }
}

// One plane: contiguous host-layout values -> pitched storage.
template <class S, class IN>
__global__ void pack_kernel(S* __restrict__ dst, const IN* __restrict__ src, int w, int h,
                            int pitch, typename Store<S>::CT wi, typename Store<S>::CT scale) {
    using CT = typename Store<S>::CT;
    const int64_t n = int64_t(w) * h;
    for (int64_t t = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; t < n;
         t += int64_t(gridDim.x) * blockDim.x) {
        const int y = int(t / w), x = int(t - int64_t(y) * w);
        dst[int64_t(y) * pitch + x] = Store<S>::enc(CT(src[t]), wi, scale);
    }
}

// One plane: pitched storage -> contiguous host-layout values.
template <class S, class OUT>
__global__ void unpack_kernel(OUT* __restrict__ dst, const S* __restrict__ src, int w, int h,
                              int pitch, typename Store<S>::CT wi,
                              typename Store<S>::CT inv_scale) {
    const int64_t n = int64_t(w) * h;
    for (int64_t t = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; t < n;
         t += int64_t(gridDim.x) * blockDim.x) {
        const int y = int(t / w), x = int(t - int64_t(y) * w);
        dst[t] = OUT(Store<S>::dec(src[int64_t(y) * pitch + x], wi, inv_scale));
    }
}

// rho, u of the stored state into f32 fields of row pitch out_pitch.
template <class S>
__global__ void moments_kernel(const S* __restrict__ f, float* __restrict__ rho,
                               float* __restrict__ ux, float* __restrict__ uy, int w, int h,
                               int pitch, int64_t plane, int out_pitch,
                               Consts<typename Store<S>::CT> c) {
    using CT = typename Store<S>::CT;
    const int64_t n = int64_t(w) * h;
    for (int64_t t = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; t < n;
         t += int64_t(gridDim.x) * blockDim.x) {
        const int y = int(t / w), x = int(t - int64_t(y) * w);
        const int64_t o = int64_t(y) * pitch + x;
        CT g[9];
#pragma unroll
        for (int i = 0; i < 9; ++i) g[i] = Store<S>::dec(f[i * plane + o], c.wt[i], c.dinv);
        CT r, vx, vy;
        cell_moments<false>(c, g, r, vx, vy);
        const int64_t q = int64_t(y) * out_pitch + x;
        rho[q] = float(r);
        ux[q] = float(vx);
        uy[q] = float(vy);
    }
}

// Solid-mask bytes -> exactly 0 or 1 (the step kernel packs them with a
// multiply that needs 0/1 bytes).
__global__ void normalize_mask_kernel(uint8_t* __restrict__ m, int w, int h, int mpitch);

// Per (row, warp tile of tile_w cells): 1 when the tile reaches a lattice
// edge that is not periodic, or has a solid cell within one cell of it (the
// general path); 2 when it reaches only periodic edges (the wrapping
// interior path); 0 otherwise (the lean interior path).
__global__ void tile_flags_kernel(uint8_t* __restrict__ tflags, const uint8_t* __restrict__ solid,
                                  int w, int h, int mpitch, int tile_w, int ntiles, int xper,
                                  int yper);

// Link masks of the tiles flagged 3 at V cells per thread: for lane l of tile
// t (cells x0 = (tile * 32 + l) * V .. x0 + V - 1 of row y), byte 0 of
// links[t * 32 + l] has bit k set when cell x0 + k is solid, and byte i
// (i = 1..8), in half-way mode, when the source cell of direction i, (y,
// x0 + k) minus the direction's displacement, is solid (that link bounces
// back).  Tiles with another flag are not written.
__global__ void link_masks_kernel(uint4* __restrict__ links, const uint8_t* __restrict__ tflags,
                                  const uint8_t* __restrict__ solid, int mpitch, int ntiles,
                                  int h, int V, int frame, int halfway);

// Sets the message lbm_last_error_string returns on this thread.
void set_last_error(const std::string& msg);

struct HealthPartial {
    double mass, mx, my, minf, mineq0;
    long long nonfinite;
};

// Per-block partial health sums; deterministic for a fixed grid size.
template <class S>
__global__ void __launch_bounds__(256)
health_kernel(const S* __restrict__ f, int w, int h, int pitch, int64_t plane,
              Consts<typename Store<S>::CT> c, HealthPartial* __restrict__ partial) {
    using CT = typename Store<S>::CT;
    using A = Ar<false>;
    double mass = 0.0, mx = 0.0, my = 0.0, minf = INFINITY, mineq = INFINITY;
    long long bad = 0;
    const int64_t n = int64_t(w) * h;
    for (int64_t t = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; t < n;
         t += int64_t(gridDim.x) * blockDim.x) {
        const int y = int(t / w), x = int(t - int64_t(y) * w);
        const int64_t o = int64_t(y) * pitch + x;
        CT g[9];
#pragma unroll
        for (int i = 0; i < 9; ++i) {
            g[i] = Store<S>::dec(f[i * plane + o], c.wt[i], c.dinv);
            if (!isfinite(double(g[i]))) ++bad;
            else minf = fmin(minf, double(g[i]));
        }
        // density / momentum in the reference order (no force term: the
        // conservation sums are of the stored state).
        CT r = A::add(CT(0), g[0]);
#pragma unroll
        for (int i = 1; i < 9; ++i) r = A::add(r, g[i]);
        CT px = A::sub(g[1], g[3]);
        px = A::add(px, g[5]);
        px = A::sub(px, g[6]);
        px = A::sub(px, g[7]);
        px = A::add(px, g[8]);
        CT py = A::sub(g[2], g[4]);
        py = A::add(py, g[5]);
        py = A::add(py, g[6]);
        py = A::sub(py, g[7]);
        py = A::sub(py, g[8]);
        mass += double(r);
        mx += double(px);
        my += double(py);
        const CT inv = A::rcp(r);
        const CT vx = A::mul(inv, px), vy = A::mul(inv, py);
        const CT v2k3 = A::mul(A::add(A::mul(vx, vx), A::mul(vy, vy)), c.k3);
        const double e0 = double(A::mul(A::mul(r, c.wt[0]), A::add(CT(1), v2k3)));
        if (!isnan(e0)) mineq = fmin(mineq, e0);
    }
    __shared__ double s_sum[3][8];
    __shared__ double s_min[2][8];
    __shared__ long long s_bad[8];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        mass += __shfl_down_sync(kFull, mass, off);
        mx += __shfl_down_sync(kFull, mx, off);
        my += __shfl_down_sync(kFull, my, off);
        minf = fmin(minf, __shfl_down_sync(kFull, minf, off));
        mineq = fmin(mineq, __shfl_down_sync(kFull, mineq, off));
        bad += __shfl_down_sync(kFull, bad, off);
    }
    if (lane == 0) {
        s_sum[0][warp] = mass; s_sum[1][warp] = mx; s_sum[2][warp] = my;
        s_min[0][warp] = minf; s_min[1][warp] = mineq; s_bad[warp] = bad;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        HealthPartial p{0.0, 0.0, 0.0, INFINITY, INFINITY, 0};
        const int nw = blockDim.x >> 5;
        for (int k = 0; k < nw; ++k) {
            p.mass += s_sum[0][k]; p.mx += s_sum[1][k]; p.my += s_sum[2][k];
            p.minf = fmin(p.minf, s_min[0][k]); p.mineq0 = fmin(p.mineq0, s_min[1][k]);
            p.nonfinite += s_bad[k];
        }
        partial[blockIdx.x] = p;
    }
}

// Reduces nblocks partials in a fixed order into out[0].
__global__ void health_final_kernel(const HealthPartial* __restrict__ partial, int nblocks,
                                    HealthPartial* __restrict__ out);

}  // namespace lbmk
