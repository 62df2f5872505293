// lbm_render.cu — the colour map of taktoa/chemsim src/render.rs on the
// device: a lattice's moments become an RGBA8 image in a headless buffer (the
// reference draws into a piston window; no graphics stack is used here).
//
//   scalar modes (render_scalar_field, src/render.rs:23-89): density or speed
//     hue 0, saturation 1, value = logistic((x - mean) / std)
//   vector modes (render_vector_field, src/render.rs:91-207): velocity or
//     momentum density (vx, vy)
//     hue = (atan2(vy, vx) + pi) / (2 pi), saturation 0.8,
//     value = logistic((m - mean) / std) with m = vx^2 + vy^2
//   then HSV -> RGB (hexcone model) and each channel = clamp(round(256 c),
//   0, 255); solid cells are painted (0, 0, 255) when the geometry overlay is
//   on (render_geometry, src/render.rs:7-21).
//
// mean and std are over every cell of the field (af::mean_all / stdev_all,
// population standard deviation), reduced in f64 in two passes with a fixed
// block order, so a render is deterministic.  The per-pixel arithmetic is
// f32 with one rounding per operation in the reference's order.
#include <algorithm>
#include <string>

#include "lbm_handle.cuh"

namespace {

constexpr int kRenderBlocks = 1024;
constexpr int kRenderThreads = 256;

struct RenderField {
    const float* rho;
    const float* ux;
    const float* uy;
    int pitch, w, h, mode;
};

// The field value whose z-score drives the image's value channel.
__device__ __forceinline__ float field_value(const RenderField& f, int64_t o) {
    switch (f.mode) {
        case LBM_RENDER_DENSITY: return f.rho[o];
        case LBM_RENDER_SPEED: {
            const float vx = f.ux[o], vy = f.uy[o];
            return __fsqrt_rn(__fadd_rn(__fmul_rn(vx, vx), __fmul_rn(vy, vy)));
        }
        case LBM_RENDER_VELOCITY: {
            const float vx = f.ux[o], vy = f.uy[o];
            return __fadd_rn(__fmul_rn(vx, vx), __fmul_rn(vy, vy));
        }
        default: {
            const float r = f.rho[o];
            const float jx = __fmul_rn(r, f.ux[o]), jy = __fmul_rn(r, f.uy[o]);
            return __fadd_rn(__fmul_rn(jx, jx), __fmul_rn(jy, jy));
        }
    }
}

// Block partial sums of x (pass 0) or (x - mean)^2 (pass 1), in f64.  Block
// b takes rows b, b + grid, ...; its threads stride along the row.
__global__ void __launch_bounds__(kRenderThreads)
render_stats_kernel(RenderField f, int pass, const double* __restrict__ mean,
                    double* __restrict__ partial) {
    const double m = pass ? *mean : 0.0;
    double acc = 0.0;
    for (int y = blockIdx.x; y < f.h; y += gridDim.x) {
        const int64_t row = int64_t(y) * f.pitch;
        for (int x = threadIdx.x; x < f.w; x += blockDim.x) {
            const double v = field_value(f, row + x);
            acc += pass ? (v - m) * (v - m) : v;
        }
    }
    __shared__ double s[kRenderThreads];
    s[threadIdx.x] = acc;
    __syncthreads();
    for (int k = kRenderThreads / 2; k > 0; k >>= 1) {
        if (threadIdx.x < k) s[threadIdx.x] += s[threadIdx.x + k];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = s[0];
}

// stats[pass] = sum of the partials / n, a fixed-order tree over one block;
// pass 1 stores the standard deviation.
__global__ void __launch_bounds__(kRenderBlocks)
render_final_kernel(const double* __restrict__ partial, int64_t n, int pass,
                    double* __restrict__ stats) {
    __shared__ double s[kRenderBlocks];
    s[threadIdx.x] = partial[threadIdx.x];
    __syncthreads();
    for (int k = kRenderBlocks / 2; k > 0; k >>= 1) {
        if (threadIdx.x < k) s[threadIdx.x] += s[threadIdx.x + k];
        __syncthreads();
    }
    if (threadIdx.x == 0) stats[pass] = pass ? sqrt(s[0] / double(n)) : s[0] / double(n);
}

// HSV -> RGB, hexcone model: sector i = floor(6h), fraction f = 6h - i.
__device__ __forceinline__ void hsv_to_rgb(float h, float s, float v, float& r, float& g,
                                           float& b) {
    const float h6 = __fmul_rn(h, 6.f);
    const int i = int(h6);
    const float fr = __fsub_rn(h6, float(i));
    const float p = __fmul_rn(v, __fsub_rn(1.f, s));
    const float q = __fmul_rn(v, __fsub_rn(1.f, __fmul_rn(fr, s)));
    const float t = __fmul_rn(v, __fsub_rn(1.f, __fmul_rn(__fsub_rn(1.f, fr), s)));
    switch (i % 6) {
        case 0: r = v; g = t; b = p; break;
        case 1: r = q; g = v; b = p; break;
        case 2: r = p; g = v; b = t; break;
        case 3: r = p; g = q; b = v; break;
        case 4: r = t; g = p; b = v; break;
        default: r = v; g = p; b = q; break;
    }
}

// (256.0 * c).round().min(255.0).max(0.0) as u8: rounds half away from zero,
// and f32::min returns the other operand for a NaN, so NaN maps to 255.
__device__ __forceinline__ unsigned char to_u8(float c) {
    const float r = roundf(__fmul_rn(256.f, c));
    if (r != r) return 255;
    return static_cast<unsigned char>(fmaxf(fminf(r, 255.f), 0.f));
}

// Clamp to [0, 1] passing NaN through (a uniform field has std 0, so its
// z-scores are 0 * inf = NaN and the pixel renders white).
__device__ __forceinline__ float clamp01(float x) { return x != x ? x : fminf(fmaxf(x, 0.f), 1.f); }

__global__ void __launch_bounds__(kRenderThreads)
render_pixels_kernel(RenderField f, const double* __restrict__ stats,
                     const uint8_t* __restrict__ solid, int mpitch, uchar4* __restrict__ out) {
    const float avg = float(stats[0]);
    const float inv_std = __fdiv_rn(1.f, float(stats[1]));
    const bool vec = f.mode == LBM_RENDER_VELOCITY || f.mode == LBM_RENDER_MOMENTUM;
    const float kPi = 3.14159265358979323846f;
    const float kHalfOverPi = __fmul_rn(0.318309886183790671538f, 0.5f);   // FRAC_1_PI * 0.5
    for (int y = blockIdx.x; y < f.h; y += gridDim.x)
    for (int x = threadIdx.x; x < f.w; x += blockDim.x) {
        const int64_t o = int64_t(y) * f.pitch + x;
        const int64_t e = int64_t(y) * f.w + x;
        uchar4 px;
        if (solid != nullptr && solid[int64_t(y) * mpitch + x]) {
            px = make_uchar4(0, 0, 255, 255);
        } else {
            const float z = __fmul_rn(__fsub_rn(field_value(f, o), avg), inv_std);
            const float val = clamp01(__fdiv_rn(1.f, __fadd_rn(1.f, expf(-z))));
            float hue = 0.f, sat = 1.f;
            if (vec) {
                float vx = f.ux[o], vy = f.uy[o];
                if (f.mode == LBM_RENDER_MOMENTUM) {
                    vx = __fmul_rn(f.rho[o], vx);
                    vy = __fmul_rn(f.rho[o], vy);
                }
                hue = clamp01(__fmul_rn(__fadd_rn(atan2f(vy, vx), kPi), kHalfOverPi));
                sat = 0.8f;
            }
            float r, g, b;
            hsv_to_rgb(hue, sat, val, r, g, b);
            px = make_uchar4(to_u8(r), to_u8(g), to_u8(b), 255);
        }
        out[e] = px;
    }
}

}  // namespace

namespace {

int cuda_status(cudaError_t e, const char* what) {
    if (e == cudaSuccess) return LBM_OK;
    (void)cudaGetLastError();
    return lbmk::lattice_fail(e == cudaErrorMemoryAllocation ? LBM_ERR_OUT_OF_MEMORY : LBM_ERR_CUDA,
                              std::string(what) + ": " + cudaGetErrorString(e));
}

// Renders into dev_out (a device image), or into the lattice's own image
// buffer when dev_out is null (returned in *img_out); all on L's stream.
int render_launch(lbm_lattice* L, int mode, int geometry_overlay, uchar4* dev_out, uchar4** img_out) {
    using lbmk::lattice_fail;
    if (mode < LBM_RENDER_DENSITY || mode > LBM_RENDER_MOMENTUM)
        return lattice_fail(LBM_ERR_INVALID_ARGUMENT, "unknown render mode");
    if (cudaSetDevice(L->dev) != cudaSuccess) return lattice_fail(LBM_ERR_CUDA, "cudaSetDevice");
    if (int rc = lbmk::lattice_refresh_moments(L)) return rc;
    const size_t img = size_t(L->w) * L->h * 4;
    const size_t need = (dev_out ? 0 : img) + (kRenderBlocks + 2) * sizeof(double);
    if (L->render_bytes < need) {
        if (L->rb_pending)                 // an asynchronous frame may still be reading it
            if (int rc = cuda_status(cudaEventSynchronize(L->rb_landed), "cudaEventSynchronize")) return rc;
        if (L->render) cudaFree(L->render);
        L->render = nullptr;
        L->render_bytes = 0;
        if (int rc = cuda_status(cudaMalloc(&L->render, need), "cudaMalloc")) return rc;
        L->render_bytes = need;
    }
    double* partial = static_cast<double*>(L->render);
    double* stats = partial + kRenderBlocks;
    uchar4* out = dev_out ? dev_out : reinterpret_cast<uchar4*>(stats + 2);
    const RenderField f{L->mom[0], L->mom[1], L->mom[2], L->pitch, L->w, L->h, mode};
    const int64_t n = int64_t(L->w) * L->h;
    for (int pass = 0; pass < 2; ++pass) {
        render_stats_kernel<<<kRenderBlocks, kRenderThreads, 0, L->stream>>>(f, pass, stats, partial);
        render_final_kernel<<<1, kRenderBlocks, 0, L->stream>>>(partial, n, pass, stats);
    }
    const int blocks = std::min(L->h, 65535 * 8);     // block b takes rows b, b + grid, ...
    render_pixels_kernel<<<blocks, kRenderThreads, 0, L->stream>>>(
        f, stats, (geometry_overlay && L->has_solid) ? L->solid : nullptr, L->mpitch, out);
    if (img_out) *img_out = out;
    return cuda_status(cudaGetLastError(), "render launch");
}

}  // namespace

extern "C" int lbm_render(lbm_lattice* L, int mode, int geometry_overlay, uint8_t* rgba,
                          int on_device) {
    using lbmk::lattice_fail;
    if (!L) return lattice_fail(LBM_ERR_INVALID_ARGUMENT, "null lattice");
    if (!rgba) return lattice_fail(LBM_ERR_INVALID_ARGUMENT, "null image pointer");
    if (L->rb_pending && !on_device)   // the lattice's image buffer may be in flight
        if (int rc = cuda_status(cudaStreamWaitEvent(L->stream, L->rb_landed, 0), "wait")) return rc;
    uchar4* out = nullptr;
    if (int rc = render_launch(L, mode, geometry_overlay,
                               on_device ? reinterpret_cast<uchar4*>(rgba) : nullptr, &out))
        return rc;
    if (!on_device)
        if (int rc = cuda_status(cudaMemcpyAsync(rgba, out, size_t(L->w) * L->h * 4,
                                                 cudaMemcpyDeviceToHost, L->stream),
                                 "cudaMemcpyAsync"))
            return rc;
    return cuda_status(cudaStreamSynchronize(L->stream), "cudaStreamSynchronize");
}

// The frame rendered on the lattice's stream, copied to the host on the
// readback stream without waiting (see lbm_read_moments_async).
extern "C" int lbm_render_async(lbm_lattice* L, int mode, int geometry_overlay, uint8_t* rgba) {
    using lbmk::lattice_fail;
    if (!L) return lattice_fail(LBM_ERR_INVALID_ARGUMENT, "null lattice");
    if (!rgba) return lattice_fail(LBM_ERR_INVALID_ARGUMENT, "null image pointer");
    if (int rc = lbmk::lattice_readback_stream(L)) return rc;
    // the image buffer is reused: its previous host copy must have finished
    if (L->rb_pending)
        if (int rc = cuda_status(cudaStreamWaitEvent(L->stream, L->rb_landed, 0), "wait")) return rc;
    uchar4* out = nullptr;
    if (int rc = render_launch(L, mode, geometry_overlay, nullptr, &out)) return rc;
    if (int rc = cuda_status(cudaEventRecord(L->rb_staged, L->stream), "record")) return rc;
    if (int rc = cuda_status(cudaStreamWaitEvent(L->rb_stream, L->rb_staged, 0), "wait")) return rc;
    if (int rc = cuda_status(cudaMemcpyAsync(rgba, out, size_t(L->w) * L->h * 4,
                                             cudaMemcpyDeviceToHost, L->rb_stream),
                             "cudaMemcpyAsync"))
        return rc;
    if (int rc = cuda_status(cudaEventRecord(L->rb_landed, L->rb_stream), "record")) return rc;
    L->rb_pending = true;
    return LBM_OK;
}
