// lbm_api.cu — the C ABI of include/lbm_cuda.h for single lattices.
//
// A handle replaces the reference's State<D2Q9> (taktoa/chemsim
// src/lbm.rs:670-819): it owns two device population buffers (A/B
// ping-pong), the solid mask, the moment buffers and one CUDA stream.
// State::step's three phases (:694-714) are one fused kernel launch per step;
// runs of steps replay a captured CUDA graph.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <type_traits>
#include <vector>

#include "lbm_aux.cuh"

using namespace lbmk;

namespace {

thread_local std::string g_err;

int fail(int code, const std::string& msg) {
    g_err = msg;
    return code;
}

int cuda_fail(cudaError_t e, const char* what) {
    (void)cudaGetLastError();   // a non-sticky error must not leak into later calls
    return fail(e == cudaErrorMemoryAllocation ? LBM_ERR_OUT_OF_MEMORY : LBM_ERR_CUDA,
                std::string(what) + ": " + cudaGetErrorString(e));
}

#define LBM_CUDA(expr)                                   \
    do {                                                 \
        cudaError_t e__ = (expr);                        \
        if (e__ != cudaSuccess) return cuda_fail(e__, #expr); \
    } while (0)

struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int dev) {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        if (prev != dev) cudaSetDevice(dev);
    }
    ~DeviceGuard() {
        if (prev >= 0) cudaSetDevice(prev);
    }
};

constexpr int kGraphSteps = 64;       // steps per captured graph (even)
constexpr int kHealthBlocks = 1024;
constexpr int kMaxSide = 65535 * 4;    // grid.y limit x 4 rows per block

size_t elem_size(int precision) {
    switch (precision) {
        case LBM_F32: return 4;
        case LBM_F64: return 8;
        case LBM_F16DEV:
        case LBM_BF16DEV: return 2;
        default: return 0;
    }
}

int default_cells(int precision) {
    switch (precision) {
        case LBM_F64: return 2;
        case LBM_F32: return 4;
        default: return 8;      // 16-bit: one 16-byte load per plane and thread
    }
}

bool valid_cells(int precision, int v) {
    switch (precision) {
        case LBM_F32: return v == 2 || v == 4 || v == 8;
        case LBM_F64: return v == 2;
        default: return v == 4 || v == 8;
    }
}

int grid_for(int64_t n, int block) {
    int64_t g = (n + block - 1) / block;
    if (g > 65535 * 8) g = 65535 * 8;
    return int(g < 1 ? 1 : g);
}

}  // namespace

#include "lbm_handle.cuh"

namespace {

// Collision constants exactly as src/lbm.rs computes them in its Scalar type
// (weights :205-215, cs :83-85, equilibrium factors :54-66, BGK :357, TRT
// :430-441).  Host code is built with -ffp-contract=off.
template <class CT>
Consts<CT> make_consts(const lbm_lattice* L) {
    Consts<CT> c{};
    const CT n[9] = {CT(16), CT(4), CT(4), CT(4), CT(4), CT(1), CT(1), CT(1), CT(1)};
    for (int i = 0; i < 9; ++i) c.wt[i] = n[i] / CT(36);
    const CT dx = CT(L->dx), dt = CT(L->dt);
    const CT cs = dx / (CT(std::sqrt(CT(3))) * dt);
    const CT cs2 = cs * cs;
    const CT cs4 = cs2 * cs2;
    c.k1 = CT(1) / cs2;
    c.k2 = CT(1) / (CT(2) * cs4);
    c.k3 = CT(-1) / (CT(2) * cs2);
    const CT tau = CT(L->tau);
    c.bgk_factor = -dt / tau;
    c.omega_p = CT(1) / tau;
    c.omega_m = CT(1) / CT(L->tau_minus);
    c.trt_scale = -dt * CT(0.5);
    c.fx = CT(L->fx);
    c.fy = CT(L->fy);
    c.hfx = c.fx * CT(0.5);
    c.hfy = c.fy * CT(0.5);
    c.guo = CT(1) - CT(1) / (CT(2) * tau);
    c.inv_cs4 = CT(1) / cs4;
    c.force = (L->fx != 0.f || L->fy != 0.f) ? 1 : 0;
    for (int i = 0; i < 9; ++i) {
        const CT cF = CT(CX(i)) * c.fx + CT(CY(i)) * c.fy;
        c.gw[i] = c.guo * c.wt[i];
        c.kcF[i] = c.k1 * cF;
        c.cF4[i] = cF * c.inv_cs4;
    }
    c.collision = L->collision;
    c.stochastic = (L->flags & LBM_ROUND_NEAREST) ? 0 : 1;
    if (L->precision == LBM_F16DEV) { c.dscale = CT(kHalfDevScale); c.dinv = CT(1) / CT(kHalfDevScale); }
    else if (L->precision == LBM_BF16DEV) { c.dscale = CT(kBf16DevScale); c.dinv = CT(1) / CT(kBf16DevScale); }
    else { c.dscale = CT(1); c.dinv = CT(1); }
    for (int i = 0; i < 9; ++i) c.sgw[i] = c.dscale * c.gw[i];
    c.shfx = c.dscale * c.hfx;
    c.shfy = c.dscale * c.hfy;
    fill_pair_consts(c);
    return c;
}

template <class S>
cudaError_t launch_one_t(lbm_lattice* L, int from, bool moments) {
    return launch_step<S>(lattice_args<S>(L, from, moments), (L->flags & LBM_FRAME_XY) ? 1 : 0,
                          (L->flags & LBM_FAST) != 0, L->vcells, L->rows, L->stream);
}

// One step whose moments go to out[0..2] (dense rows of w elements).
template <class S>
cudaError_t launch_to_t(lbm_lattice* L, float* const* out) {
    StepArgs<typename Store<S>::CT> a = lattice_args<S>(L, L->cur, false);
    a.mom_rho = out[0];
    a.mom_ux = out[1];
    a.mom_uy = out[2];
    a.mom_pitch = L->w;
    return launch_step<S>(a, (L->flags & LBM_FRAME_XY) ? 1 : 0, (L->flags & LBM_FAST) != 0,
                          L->vcells, L->rows, L->stream);
}

cudaError_t launch_one_to(lbm_lattice* L, float* const* out) {
    switch (L->precision) {
        case LBM_F32: return launch_to_t<float>(L, out);
        case LBM_F64: return launch_to_t<double>(L, out);
        case LBM_F16DEV: return launch_to_t<__half>(L, out);
        default: return launch_to_t<__nv_bfloat16>(L, out);
    }
}

cudaError_t launch_one(lbm_lattice* L, int from, bool moments) {
    switch (L->precision) {
        case LBM_F32: return launch_one_t<float>(L, from, moments);
        case LBM_F64: return launch_one_t<double>(L, from, moments);
        case LBM_F16DEV: return launch_one_t<__half>(L, from, moments);
        default: return launch_one_t<__nv_bfloat16>(L, from, moments);
    }
}

void drop_graphs(lbm_lattice* L) {
    for (auto& g : L->graph) {
        if (g) cudaGraphExecDestroy(g);
        g = nullptr;
    }
}

// Captures the kGraphSteps-step graph that starts from buffer `start`.
int ensure_graph(lbm_lattice* L, int start) {
    if (L->dirty) { drop_graphs(L); L->dirty = false; }
    if (L->graph[start]) return LBM_OK;
    LBM_CUDA(cudaStreamBeginCapture(L->stream, cudaStreamCaptureModeThreadLocal));
    int from = start;
    cudaError_t err = cudaSuccess;
    for (int s = 0; s < kGraphSteps && err == cudaSuccess; ++s) {
        err = launch_one(L, from, false);
        from ^= 1;
    }
    cudaGraph_t g = nullptr;
    cudaError_t e2 = cudaStreamEndCapture(L->stream, &g);
    if (err != cudaSuccess) { if (g) cudaGraphDestroy(g); return cuda_fail(err, "step capture"); }
    if (e2 != cudaSuccess) return cuda_fail(e2, "cudaStreamEndCapture");
    cudaError_t e3 = cudaGraphInstantiate(&L->graph[start], g, 0);
    cudaGraphDestroy(g);
    if (e3 != cudaSuccess) { L->graph[start] = nullptr; return cuda_fail(e3, "cudaGraphInstantiate"); }
    return LBM_OK;
}

int ensure_staging(lbm_lattice* L, size_t bytes) {
    if (L->staging_bytes >= bytes) return LBM_OK;
    if (L->staging) cudaFree(L->staging);
    L->staging = nullptr;
    L->staging_bytes = 0;
    LBM_CUDA(cudaMalloc(&L->staging, bytes));
    L->staging_bytes = bytes;
    return LBM_OK;
}

#ifndef LBM_LINKS_IN_GRID
#define LBM_LINKS_IN_GRID 1
#endif

// Recomputes the per-(row, warp tile) boundary/solid flags for the current
// tile width and geometry.
int refresh_tiles(lbm_lattice* L) {
    const int tile_w = 32 * L->vcells;
    L->ntiles = (L->w + tile_w - 1) / tile_w;
    const int64_t n = int64_t(L->h) * L->ntiles;
    // Edge tiles of periodic axes only need wrapped addresses: the interior
    // path takes them.
    const int xper = (L->flags & 3) == LBM_X_PERIODIC ? 1 : 0;
    const int yper = ((L->flags >> 2) & 3) == 1 ? 1 : 0;
    tile_flags_kernel<<<grid_for(n, 256), 256, 0, L->stream>>>(
        L->tflags, L->has_solid ? L->solid : nullptr, L->w, L->h, L->mpitch, tile_w, L->ntiles,
        xper, yper);
    LBM_CUDA(cudaGetLastError());
    // Compact the flagged tiles on the host (row-major order, deterministic).
    std::vector<uint8_t> flags(static_cast<size_t>(n));
    LBM_CUDA(cudaMemcpyAsync(flags.data(), L->tflags, flags.size(), cudaMemcpyDeviceToHost,
                             L->stream));
    LBM_CUDA(cudaStreamSynchronize(L->stream));
    // 16-bit storage at 8 cells per thread and f32 at any tile width: tiles
    // flagged 3 take the interior path with per-lane link masks (computed
    // here), so only tiles flagged 1 are listed.
    const bool dev16 = L->precision == LBM_F16DEV || L->precision == LBM_BF16DEV;
    const bool in_grid = LBM_LINKS_IN_GRID && L->has_solid &&
                         ((dev16 && L->vcells == 8) || (LBM_LINKS_F32 && L->precision == LBM_F32));
    if (in_grid) {
        const size_t need = size_t(n) * 32;
        if (need > L->links_cap) {
            if (L->links) cudaFree(L->links);
            L->links = nullptr;
            L->links_cap = 0;
            LBM_CUDA(cudaMalloc(reinterpret_cast<void**>(&L->links), need * sizeof(uint4)));
            L->links_cap = need;
        }
        link_masks_kernel<<<grid_for(int64_t(need), 256), 256, 0, L->stream>>>(
            L->links, L->tflags, L->solid, L->mpitch, L->ntiles, L->h, L->vcells,
            (L->flags & LBM_FRAME_XY) ? 1 : 0, (L->flags & LBM_SOLID_HALFWAY) ? 1 : 0);
        LBM_CUDA(cudaGetLastError());
    }
    L->use_links = in_grid;
    // Entries of tiles flagged 3 carry bit 31 (the general path without edge
    // handling); row * ntiles + tile stays below 2^31 (h <= 65535 * 8 rows).
    std::vector<uint32_t> list;
    for (int64_t t = 0; t < n; ++t) {
        const uint8_t f = flags[size_t(t)];
        if (f == 1) list.push_back(uint32_t(t));
        else if (f == 3 && !in_grid) list.push_back(uint32_t(t) | 0x80000000u);
    }
    if (list.size() > L->gtiles_cap) {
        if (L->gtiles) cudaFree(L->gtiles);
        L->gtiles = nullptr;
        L->gtiles_cap = 0;
        LBM_CUDA(cudaMalloc(reinterpret_cast<void**>(&L->gtiles), list.size() * sizeof(uint32_t)));
        L->gtiles_cap = list.size();
    }
    if (!list.empty())
        LBM_CUDA(cudaMemcpyAsync(L->gtiles, list.data(), list.size() * sizeof(uint32_t),
                                 cudaMemcpyHostToDevice, L->stream));
    LBM_CUDA(cudaStreamSynchronize(L->stream));
    L->ngtiles = int(list.size());
    L->dirty = true;
    ++L->version;
    return LBM_OK;
}

template <class S, class IN>
int set_pops_t(lbm_lattice* L, const IN* f) {
    using CT = typename Store<S>::CT;
    const Consts<CT> c = make_consts<CT>(L);
    const int64_t n = int64_t(L->w) * L->h;
    S* dst = static_cast<S*>(L->buf[L->cur]);
    if constexpr (std::is_same<S, IN>::value) {
        for (int i = 0; i < 9; ++i)
            LBM_CUDA(cudaMemcpy2DAsync(dst + i * L->plane, size_t(L->pitch) * sizeof(S), f + i * n,
                                       size_t(L->w) * sizeof(IN), size_t(L->w) * sizeof(IN), L->h,
                                       cudaMemcpyHostToDevice, L->stream));
    } else {
        int rc = ensure_staging(L, size_t(n) * sizeof(IN));
        if (rc) return rc;
        IN* st = static_cast<IN*>(L->staging);
        for (int i = 0; i < 9; ++i) {
            LBM_CUDA(cudaMemcpyAsync(st, f + i * n, size_t(n) * sizeof(IN), cudaMemcpyHostToDevice,
                                     L->stream));
            pack_kernel<S, IN><<<grid_for(n, 256), 256, 0, L->stream>>>(
                dst + i * L->plane, st, L->w, L->h, L->pitch, c.wt[i], c.dscale);
            LBM_CUDA(cudaGetLastError());
        }
    }
    LBM_CUDA(cudaStreamSynchronize(L->stream));
    return LBM_OK;
}

template <class S, class OUT>
int get_pops_t(lbm_lattice* L, OUT* f) {
    using CT = typename Store<S>::CT;
    const Consts<CT> c = make_consts<CT>(L);
    const int64_t n = int64_t(L->w) * L->h;
    const S* src = static_cast<const S*>(L->buf[L->cur]);
    if constexpr (std::is_same<S, OUT>::value) {
        for (int i = 0; i < 9; ++i)
            LBM_CUDA(cudaMemcpy2DAsync(f + i * n, size_t(L->w) * sizeof(OUT), src + i * L->plane,
                                       size_t(L->pitch) * sizeof(S), size_t(L->w) * sizeof(OUT),
                                       L->h, cudaMemcpyDeviceToHost, L->stream));
    } else {
        int rc = ensure_staging(L, size_t(n) * sizeof(OUT));
        if (rc) return rc;
        OUT* st = static_cast<OUT*>(L->staging);
        for (int i = 0; i < 9; ++i) {
            unpack_kernel<S, OUT><<<grid_for(n, 256), 256, 0, L->stream>>>(
                st, src + i * L->plane, L->w, L->h, L->pitch, c.wt[i], c.dinv);
            LBM_CUDA(cudaGetLastError());
            LBM_CUDA(cudaMemcpyAsync(f + i * n, st, size_t(n) * sizeof(OUT), cudaMemcpyDeviceToHost,
                                     L->stream));
        }
    }
    LBM_CUDA(cudaStreamSynchronize(L->stream));
    return LBM_OK;
}

template <class S>
int eq_init_t(lbm_lattice* L) {
    using CT = typename Store<S>::CT;
    const int64_t n = int64_t(L->w) * L->h;
    eq_init_kernel<S><<<grid_for(n, 256), 256, 0, L->stream>>>(
        static_cast<S*>(L->buf[L->cur]), L->mom[0], L->mom[1], L->mom[2], L->w, L->h, L->pitch,
        L->plane, make_consts<CT>(L));
    LBM_CUDA(cudaGetLastError());
    return LBM_OK;
}

template <class S>
int fill_rest_t(lbm_lattice* L, int which) {
    using CT = typename Store<S>::CT;
    fill_rest_kernel<S><<<grid_for(L->plane, 256), 256, 0, L->stream>>>(
        static_cast<S*>(L->buf[which]), L->plane, make_consts<CT>(L));
    LBM_CUDA(cudaGetLastError());
    return LBM_OK;
}

template <class S>
int moments_t(lbm_lattice* L) {
    using CT = typename Store<S>::CT;
    const int64_t n = int64_t(L->w) * L->h;
    moments_kernel<S><<<grid_for(n, 256), 256, 0, L->stream>>>(
        static_cast<const S*>(L->buf[L->cur]), L->mom[0], L->mom[1], L->mom[2], L->w, L->h,
        L->pitch, L->plane, L->pitch, make_consts<CT>(L));
    LBM_CUDA(cudaGetLastError());
    return LBM_OK;
}

template <class S>
int health_t(lbm_lattice* L) {
    using CT = typename Store<S>::CT;
    health_kernel<S><<<kHealthBlocks, 256, 0, L->stream>>>(
        static_cast<const S*>(L->buf[L->cur]), L->w, L->h, L->pitch, L->plane,
        make_consts<CT>(L), L->health);
    LBM_CUDA(cudaGetLastError());
    health_final_kernel<<<1, 32, 0, L->stream>>>(L->health, kHealthBlocks, L->health + kHealthBlocks);
    LBM_CUDA(cudaGetLastError());
    return LBM_OK;
}

#define LBM_DISPATCH(L, fn, ...)                                        \
    ((L)->precision == LBM_F32    ? fn<float>(__VA_ARGS__)              \
     : (L)->precision == LBM_F64  ? fn<double>(__VA_ARGS__)             \
     : (L)->precision == LBM_F16DEV ? fn<__half>(__VA_ARGS__)           \
                                    : fn<__nv_bfloat16>(__VA_ARGS__))

int check_handle(const lbm_lattice* L) {
    if (!L) return fail(LBM_ERR_INVALID_ARGUMENT, "null lattice handle");
    return LBM_OK;
}

int steps_impl(lbm_lattice* L, int nsteps, bool moments) {
    if (nsteps < 0) return fail(LBM_ERR_INVALID_ARGUMENT, "nsteps must be >= 0");
    if (nsteps == 0) return LBM_OK;
    const int plain = moments ? nsteps - 1 : nsteps;
    const int full = plain / kGraphSteps;
    const int rem = plain % kGraphSteps;
    // The graphs of both buffer parities are captured at the first step call
    // after any change of the step arguments, so a long run that follows a
    // few short ones does not pay for the capture.
    // While the caller captures the stream into a graph of its own, the
    // steps are plain launches (captured there).
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    LBM_CUDA(cudaStreamIsCapturing(L->stream, &cap));
    const bool capturing = cap != cudaStreamCaptureStatusNone;
    if (!capturing)
        for (int p = 0; p < 2; ++p)
            if (int rc = ensure_graph(L, p)) return rc;
    for (int k = 0; k < full; ++k) {
        if (capturing) {
            for (int s = 0; s < kGraphSteps; ++s) {
                LBM_CUDA(launch_one(L, L->cur, false));
                L->cur ^= 1;
            }
        } else {
            LBM_CUDA(cudaGraphLaunch(L->graph[L->cur], L->stream));
        }
    }
    for (int k = 0; k < rem; ++k) {
        LBM_CUDA(launch_one(L, L->cur, false));
        L->cur ^= 1;
    }
    if (moments) {
        LBM_CUDA(launch_one(L, L->cur, true));
        L->cur ^= 1;
    }
    // State::step: time += delta_t once per step, in f32 (src/lbm.rs:713).
    for (int k = 0; k < nsteps; ++k) L->time += L->dt;
    L->steps += nsteps;
    L->mom_valid = moments;
    return LBM_OK;
}

}  // namespace

namespace lbmk {
void set_last_error(const std::string& msg) { g_err = msg; }

int lattice_fail(int code, const std::string& msg) { return fail(code, msg); }

template <class S>
StepArgs<typename Store<S>::CT> lattice_args(const lbm_lattice* L, int from, bool moments) {
    using CT = typename Store<S>::CT;
    StepArgs<CT> a{};
    a.src = L->buf[from];
    a.dst = L->buf[from ^ 1];
    a.solid = L->has_solid ? L->solid : nullptr;
    a.tflags = L->tflags;
    a.ntiles = L->ntiles;
    a.gtiles = L->gtiles;
    a.ngtiles = L->ngtiles;
    a.links = L->use_links ? L->links : nullptr;
    if (moments) { a.mom_rho = L->mom[0]; a.mom_ux = L->mom[1]; a.mom_uy = L->mom[2]; }
    a.mom_pitch = L->pitch;
    a.w = L->w; a.h = L->h; a.pitch = L->pitch; a.mpitch = L->mpitch; a.plane = L->plane;
    a.flags = L->flags;
    a.pf_rows = -1;          // the launcher sizes the L2 prefetch distance
    a.c = make_consts<CT>(L);
    return a;
}
template StepArgs<float> lattice_args<float>(const lbm_lattice*, int, bool);
template StepArgs<double> lattice_args<double>(const lbm_lattice*, int, bool);
template StepArgs<float> lattice_args<__half>(const lbm_lattice*, int, bool);
template StepArgs<float> lattice_args<__nv_bfloat16>(const lbm_lattice*, int, bool);

int lattice_refresh_moments(lbm_lattice* L) {
    if (L->mom_valid) return LBM_OK;
    DeviceGuard g(L->dev);
    if (int rc = LBM_DISPATCH(L, moments_t, L)) return rc;
    L->mom_valid = true;
    return LBM_OK;
}

int lattice_readback_stream(lbm_lattice* L) {
    if (L->rb_stream) return LBM_OK;
    DeviceGuard g(L->dev);
    LBM_CUDA(cudaStreamCreateWithFlags(&L->rb_stream, cudaStreamNonBlocking));
    LBM_CUDA(cudaEventCreateWithFlags(&L->rb_staged, cudaEventDisableTiming));
    LBM_CUDA(cudaEventCreateWithFlags(&L->rb_landed, cudaEventDisableTiming));
    for (auto& e : L->rb_done) LBM_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    return LBM_OK;
}

void lattice_advance(lbm_lattice* L, int nsteps) {
    if (nsteps & 1) L->cur ^= 1;
    for (int k = 0; k < nsteps; ++k) L->time += L->dt;
    L->steps += nsteps;
    L->mom_valid = false;
}

__global__ void normalize_mask_kernel(uint8_t* __restrict__ m, int w, int h, int mpitch) {
    const int64_t n = int64_t(w) * h;
    for (int64_t t = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; t < n;
         t += int64_t(gridDim.x) * blockDim.x) {
        const int y = int(t / w), x = int(t - int64_t(y) * w);
        uint8_t* p = m + int64_t(y) * mpitch + x;
        *p = *p != 0;
    }
}

__global__ void tile_flags_kernel(uint8_t* __restrict__ tflags, const uint8_t* __restrict__ solid,
                                  int w, int h, int mpitch, int tile_w, int ntiles, int xper,
                                  int yper) {
    const int64_t n = int64_t(h) * ntiles;
    for (int64_t t = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; t < n;
         t += int64_t(gridDim.x) * blockDim.x) {
        const int y = int(t / ntiles), tt = int(t - int64_t(y) * ntiles);
        const int xs = tt * tile_w;
        const bool xedge = xs == 0 || xs + tile_w >= w;
        const bool yedge = y == 0 || y == h - 1;
        bool gen = (xedge && !xper) || (yedge && !yper);
        bool solid_gen = false;
        if (!gen && solid != nullptr) {
            const int xe = min(xs + tile_w, w);          // columns xs-1 .. xe, wrapped
            for (int r = y - 1; r <= y + 1 && !gen; ++r) {
                const int rr = r < 0 ? r + h : (r >= h ? r - h : r);
                const uint8_t* row = solid + int64_t(rr) * mpitch;
                for (int c = xs - 1; c <= xe; ++c) {
                    const int cc = c < 0 ? c + w : (c >= w ? c - w : c);
                    if (row[cc]) { gen = solid_gen = true; break; }
                }
            }
        }
        // 3: solids nearby but every source cell inside the lattice (the
        // general path without edge handling); 1: the full general path
        // Unlisted tiles: 2 for the partial last tile of a periodic row (the
        // wrapping path), 0 otherwise (the interior path wraps rows and its
        // edge columns at periodic edges itself).
        tflags[t] = gen ? ((solid_gen && !xedge && !yedge) ? 3 : 1) : ((xs + tile_w > w) ? 2 : 0);
    }
}

__global__ void link_masks_kernel(uint4* __restrict__ links, const uint8_t* __restrict__ tflags,
                                  const uint8_t* __restrict__ solid, int mpitch, int ntiles,
                                  int h, int V, int frame, int halfway) {
    const int64_t n = int64_t(h) * ntiles * 32;
    for (int64_t q = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; q < n;
         q += int64_t(gridDim.x) * blockDim.x) {
        const int64_t t = q >> 5;
        if (tflags[t] != 3) continue;
        const int y = int(t / ntiles), tile = int(t - int64_t(y) * ntiles);
        const int x0 = (tile * 32 + int(q & 31)) * V;
        // a tile flagged 3 reaches no lattice edge: rows y - 1 .. y + 1 and
        // columns x0 - 1 .. x0 + V are inside the lattice
        uint32_t b[9] = {0u, 0u, 0u, 0u, 0u, 0u, 0u, 0u, 0u};
        for (int k = 0; k < V; ++k) {
            const int x = x0 + k;
            b[0] |= uint32_t(solid[int64_t(y) * mpitch + x] != 0) << k;
            if (!halfway) continue;
            for (int i = 1; i < 9; ++i) {
                const int sy = y - DROW(frame, i), sx = x - DCOL(frame, i);
                b[i] |= uint32_t(solid[int64_t(sy) * mpitch + sx] != 0) << k;
            }
        }
        uint4 o;
        o.x = b[0] | (b[1] << 8) | (b[2] << 16) | (b[3] << 24);
        o.y = b[4] | (b[5] << 8) | (b[6] << 16) | (b[7] << 24);
        o.z = b[8];
        o.w = 0u;
        links[q] = o;
    }
}

__global__ void health_final_kernel(const HealthPartial* __restrict__ partial, int nblocks,
                                    HealthPartial* __restrict__ out) {
    if (threadIdx.x != 0) return;
    HealthPartial p{0.0, 0.0, 0.0, INFINITY, INFINITY, 0};
    for (int k = 0; k < nblocks; ++k) {
        p.mass += partial[k].mass;
        p.mx += partial[k].mx;
        p.my += partial[k].my;
        p.minf = fmin(p.minf, partial[k].minf);
        p.mineq0 = fmin(p.mineq0, partial[k].mineq0);
        p.nonfinite += partial[k].nonfinite;
    }
    *out = p;
}
}  // namespace lbmk

extern "C" {

const char* lbm_last_error_string(void) { return g_err.c_str(); }

int lbm_version(void) { return 100; }

int lbm_create(int w, int h, float tau, int precision, int flags, lbm_lattice** out) {
    if (!out) return fail(LBM_ERR_INVALID_ARGUMENT, "out must not be null");
    *out = nullptr;
    if (w < 1 || h < 1 || w > kMaxSide || h > kMaxSide)
        return fail(LBM_ERR_INVALID_ARGUMENT, "lattice sides must be in [1, 262140]");
    if (!(tau > 0.f) || !std::isfinite(tau))
        return fail(LBM_ERR_INVALID_ARGUMENT, "tau must be finite and > 0");
    const size_t es = elem_size(precision);
    if (!es) return fail(LBM_ERR_INVALID_ARGUMENT, "unknown precision");
    if ((flags & 3) == 3 || ((flags >> 2) & 3) == 3 || (flags & ~0xff))
        return fail(LBM_ERR_INVALID_ARGUMENT, "invalid boundary flags");
    int dev = 0;
    LBM_CUDA(cudaGetDevice(&dev));
    lbm_lattice* L = new lbm_lattice();
    L->w = w; L->h = h; L->precision = precision; L->flags = flags; L->tau = tau;
    L->esize = es;
    L->dev = dev;
    const int per128 = int(128 / es);
    L->pitch = (w + per128 - 1) / per128 * per128;
    L->mpitch = (w + 127) / 128 * 128;
    L->plane = int64_t(L->pitch) * h;
    L->vcells = default_cells(precision);
    L->rows = 4;
    auto cleanup = [&](int rc) { lbm_destroy(L); return rc; };
    cudaError_t e;
    for (int b = 0; b < 2; ++b) {
        e = cudaMalloc(&L->buf[b], size_t(9) * L->plane * es);
        if (e != cudaSuccess) return cleanup(cuda_fail(e, "population buffer"));
    }
    for (int m = 0; m < 3; ++m) {
        e = cudaMalloc(reinterpret_cast<void**>(&L->mom[m]), size_t(L->plane) * sizeof(float));
        if (e != cudaSuccess) return cleanup(cuda_fail(e, "moment buffer"));
    }
    e = cudaMalloc(reinterpret_cast<void**>(&L->health), sizeof(HealthPartial) * (kHealthBlocks + 1));
    if (e != cudaSuccess) return cleanup(cuda_fail(e, "health scratch"));
    e = cudaMalloc(reinterpret_cast<void**>(&L->tflags), size_t(h) * ((w + 31) / 32));
    if (e != cudaSuccess) return cleanup(cuda_fail(e, "tile flags"));
    e = cudaStreamCreateWithFlags(&L->own, cudaStreamNonBlocking);
    if (e != cudaSuccess) return cleanup(cuda_fail(e, "stream"));
    L->stream = L->own;
    for (int b = 0; b < 2; ++b) {
        int rc = LBM_DISPATCH(L, fill_rest_t, L, b);
        if (rc) return cleanup(rc);
    }
    if (int rc = refresh_tiles(L)) return cleanup(rc);
    e = cudaStreamSynchronize(L->stream);
    if (e != cudaSuccess) return cleanup(cuda_fail(e, "create"));
    *out = L;
    return LBM_OK;
}

int lbm_destroy(lbm_lattice* L) {
    if (!L) return LBM_OK;
    {
        DeviceGuard g(L->dev);
        if (L->stream) cudaStreamSynchronize(L->stream);
        drop_graphs(L);
        for (auto& b : L->buf) if (b) cudaFree(b);
        for (auto& m : L->mom) if (m) cudaFree(m);
        if (L->solid) cudaFree(L->solid);
        if (L->staging) cudaFree(L->staging);
        if (L->health) cudaFree(L->health);
        if (L->render) cudaFree(L->render);
        if (L->rb_stream) cudaStreamSynchronize(L->rb_stream);
        for (auto& b : L->rb) if (b) cudaFree(b);
        if (L->rb_stream) cudaStreamDestroy(L->rb_stream);
        if (L->rb_staged) cudaEventDestroy(L->rb_staged);
        if (L->rb_landed) cudaEventDestroy(L->rb_landed);
        for (auto& e : L->rb_done) if (e) cudaEventDestroy(e);
        if (L->tflags) cudaFree(L->tflags);
        if (L->gtiles) cudaFree(L->gtiles);
        if (L->links) cudaFree(L->links);
        if (L->own) cudaStreamDestroy(L->own);
    }
    delete L;
    return LBM_OK;
}

int lbm_set_discretization(lbm_lattice* L, float dx, float dt) {
    if (int rc = check_handle(L)) return rc;
    if (!(dx > 0.f) || !(dt > 0.f) || !std::isfinite(dx) || !std::isfinite(dt))
        return fail(LBM_ERR_INVALID_ARGUMENT, "delta_x and delta_t must be finite and > 0");
    L->dx = dx; L->dt = dt; L->dirty = true; ++L->version; L->mom_valid = false;
    return LBM_OK;
}

int lbm_set_collision(lbm_lattice* L, int kind, float tau, float tau_minus) {
    if (int rc = check_handle(L)) return rc;
    if (kind != LBM_COLLISION_BGK && kind != LBM_COLLISION_TRT)
        return fail(LBM_ERR_INVALID_ARGUMENT, "unknown collision operator");
    if (!(tau > 0.f) || !std::isfinite(tau))
        return fail(LBM_ERR_INVALID_ARGUMENT, "tau must be finite and > 0");
    if (kind == LBM_COLLISION_TRT && (!(tau_minus > 0.f) || !std::isfinite(tau_minus)))
        return fail(LBM_ERR_INVALID_ARGUMENT, "tau_minus must be finite and > 0");
    L->collision = kind; L->tau = tau;
    L->tau_minus = kind == LBM_COLLISION_TRT ? tau_minus : 1.f;
    L->dirty = true;
    ++L->version;
    return LBM_OK;
}

int lbm_init_equilibrium(lbm_lattice* L, const float* rho, const float* ux, const float* uy) {
    if (int rc = check_handle(L)) return rc;
    if (!rho || !ux || !uy) return fail(LBM_ERR_INVALID_ARGUMENT, "null field pointer");
    DeviceGuard g(L->dev);
    const float* src[3] = {rho, ux, uy};
    for (int m = 0; m < 3; ++m)
        LBM_CUDA(cudaMemcpy2DAsync(L->mom[m], size_t(L->pitch) * 4, src[m], size_t(L->w) * 4,
                                   size_t(L->w) * 4, L->h, cudaMemcpyHostToDevice, L->stream));
    if (int rc = LBM_DISPATCH(L, eq_init_t, L)) return rc;
    LBM_CUDA(cudaStreamSynchronize(L->stream));
    L->mom_valid = false;
    return LBM_OK;
}

int lbm_set_populations(lbm_lattice* L, const float* f) {
    if (int rc = check_handle(L)) return rc;
    if (!f) return fail(LBM_ERR_INVALID_ARGUMENT, "null population pointer");
    DeviceGuard g(L->dev);
    L->mom_valid = false;
    switch (L->precision) {
        case LBM_F32: return set_pops_t<float, float>(L, f);
        case LBM_F64: return set_pops_t<double, float>(L, f);
        case LBM_F16DEV: return set_pops_t<__half, float>(L, f);
        default: return set_pops_t<__nv_bfloat16, float>(L, f);
    }
}

int lbm_get_populations(lbm_lattice* L, float* f) {
    if (int rc = check_handle(L)) return rc;
    if (!f) return fail(LBM_ERR_INVALID_ARGUMENT, "null population pointer");
    DeviceGuard g(L->dev);
    switch (L->precision) {
        case LBM_F32: return get_pops_t<float, float>(L, f);
        case LBM_F64: return get_pops_t<double, float>(L, f);
        case LBM_F16DEV: return get_pops_t<__half, float>(L, f);
        default: return get_pops_t<__nv_bfloat16, float>(L, f);
    }
}

int lbm_set_populations_f64(lbm_lattice* L, const double* f) {
    if (int rc = check_handle(L)) return rc;
    if (!f) return fail(LBM_ERR_INVALID_ARGUMENT, "null population pointer");
    DeviceGuard g(L->dev);
    L->mom_valid = false;
    switch (L->precision) {
        case LBM_F32: return set_pops_t<float, double>(L, f);
        case LBM_F64: return set_pops_t<double, double>(L, f);
        case LBM_F16DEV: return set_pops_t<__half, double>(L, f);
        default: return set_pops_t<__nv_bfloat16, double>(L, f);
    }
}

int lbm_get_populations_f64(lbm_lattice* L, double* f) {
    if (int rc = check_handle(L)) return rc;
    if (!f) return fail(LBM_ERR_INVALID_ARGUMENT, "null population pointer");
    DeviceGuard g(L->dev);
    switch (L->precision) {
        case LBM_F32: return get_pops_t<float, double>(L, f);
        case LBM_F64: return get_pops_t<double, double>(L, f);
        case LBM_F16DEV: return get_pops_t<__half, double>(L, f);
        default: return get_pops_t<__nv_bfloat16, double>(L, f);
    }
}

int lbm_set_geometry(lbm_lattice* L, const uint8_t* solid) {
    if (int rc = check_handle(L)) return rc;
    DeviceGuard g(L->dev);
    if (!solid) {
        if (L->has_solid) {
            L->has_solid = false;
            if (int rc = refresh_tiles(L)) return rc;
            LBM_CUDA(cudaStreamSynchronize(L->stream));
        }
        return LBM_OK;
    }
    if (!L->solid) {
        LBM_CUDA(cudaMalloc(reinterpret_cast<void**>(&L->solid), size_t(L->mpitch) * L->h));
        LBM_CUDA(cudaMemsetAsync(L->solid, 0, size_t(L->mpitch) * L->h, L->stream));
    }
    LBM_CUDA(cudaMemcpy2DAsync(L->solid, L->mpitch, solid, L->w, L->w, L->h,
                               cudaMemcpyHostToDevice, L->stream));
    normalize_mask_kernel<<<grid_for(int64_t(L->w) * L->h, 256), 256, 0, L->stream>>>(
        L->solid, L->w, L->h, L->mpitch);
    LBM_CUDA(cudaGetLastError());
    L->has_solid = true;
    if (int rc = refresh_tiles(L)) return rc;
    LBM_CUDA(cudaStreamSynchronize(L->stream));
    return LBM_OK;
}

int lbm_set_force(lbm_lattice* L, float fx, float fy) {
    if (int rc = check_handle(L)) return rc;
    if (!std::isfinite(fx) || !std::isfinite(fy))
        return fail(LBM_ERR_INVALID_ARGUMENT, "force must be finite");
    L->fx = fx; L->fy = fy; L->dirty = true; ++L->version; L->mom_valid = false;
    return LBM_OK;
}

int lbm_step(lbm_lattice* L, int nsteps) {
    if (int rc = check_handle(L)) return rc;
    DeviceGuard g(L->dev);
    return steps_impl(L, nsteps, false);
}

int lbm_step_moments(lbm_lattice* L, int nsteps) {
    if (int rc = check_handle(L)) return rc;
    if (nsteps < 1) return fail(LBM_ERR_INVALID_ARGUMENT, "lbm_step_moments needs nsteps >= 1");
    DeviceGuard g(L->dev);
    return steps_impl(L, nsteps, true);
}

int lbm_read_moments(lbm_lattice* L, float* rho, float* ux, float* uy, int on_device) {
    if (int rc = check_handle(L)) return rc;
    if (!rho || !ux || !uy) return fail(LBM_ERR_INVALID_ARGUMENT, "null field pointer");
    DeviceGuard g(L->dev);
    if (!L->mom_valid) {
        if (int rc = LBM_DISPATCH(L, moments_t, L)) return rc;
        L->mom_valid = true;
    }
    float* dst[3] = {rho, ux, uy};
    const cudaMemcpyKind kind = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    for (int m = 0; m < 3; ++m)
        LBM_CUDA(cudaMemcpy2DAsync(dst[m], size_t(L->w) * 4, L->mom[m], size_t(L->pitch) * 4,
                                   size_t(L->w) * 4, L->h, kind, L->stream));
    LBM_CUDA(cudaStreamSynchronize(L->stream));
    return LBM_OK;
}

int lbm_read_moments_async(lbm_lattice* L, float* rho, float* ux, float* uy) {
    if (int rc = check_handle(L)) return rc;
    if (!rho || !ux || !uy) return fail(LBM_ERR_INVALID_ARGUMENT, "null field pointer");
    DeviceGuard g(L->dev);
    const size_t plane = size_t(L->w) * L->h;
    if (int rc = lattice_readback_stream(L)) return rc;
    if (!L->rb[0]) {
        // both staging areas at once, so no later call allocates
        if (L->rb_pending) LBM_CUDA(cudaEventSynchronize(L->rb_landed));
        for (auto& b : L->rb) LBM_CUDA(cudaMalloc(reinterpret_cast<void**>(&b), 3 * plane * sizeof(float)));
    }
    if (!L->mom_valid) {
        if (int rc = LBM_DISPATCH(L, moments_t, L)) return rc;
        L->mom_valid = true;
    }
    // Two staging areas in turn: this one's previous host copy must have
    // finished; the other one's may still run while this one is staged and
    // the next steps run.
    const int i = L->rb_next;
    L->rb_next ^= 1;
    float* rb = L->rb[i];
    if (L->rb_used[i]) LBM_CUDA(cudaStreamWaitEvent(L->stream, L->rb_done[i], 0));
    for (int m = 0; m < 3; ++m)
        LBM_CUDA(cudaMemcpy2DAsync(rb + m * plane, size_t(L->w) * 4, L->mom[m],
                                   size_t(L->pitch) * 4, size_t(L->w) * 4, L->h,
                                   cudaMemcpyDeviceToDevice, L->stream));
    LBM_CUDA(cudaEventRecord(L->rb_staged, L->stream));
    LBM_CUDA(cudaStreamWaitEvent(L->rb_stream, L->rb_staged, 0));
    float* dst[3] = {rho, ux, uy};
    for (int m = 0; m < 3; ++m)
        LBM_CUDA(cudaMemcpyAsync(dst[m], rb + m * plane, plane * sizeof(float),
                                 cudaMemcpyDeviceToHost, L->rb_stream));
    LBM_CUDA(cudaEventRecord(L->rb_done[i], L->rb_stream));
    L->rb_used[i] = true;
    // the copy stream is in order: the latest landing covers every earlier one
    LBM_CUDA(cudaEventRecord(L->rb_landed, L->rb_stream));
    L->rb_pending = true;
    return LBM_OK;
}

int lbm_step_moments_to(lbm_lattice* L, int nsteps, float* rho, float* ux, float* uy) {
    if (int rc = check_handle(L)) return rc;
    if (nsteps < 1) return fail(LBM_ERR_INVALID_ARGUMENT, "lbm_step_moments_to needs nsteps >= 1");
    if (!rho || !ux || !uy) return fail(LBM_ERR_INVALID_ARGUMENT, "null field pointer");
    DeviceGuard g(L->dev);
    // Only memory the GPU can address is accepted: device or managed
    // allocations, and pinned host memory (its device alias is used).
    float* out[3] = {rho, ux, uy};
    for (int m = 0; m < 3; ++m) {
        cudaPointerAttributes at{};
        cudaError_t e = cudaPointerGetAttributes(&at, out[m]);
        if (e != cudaSuccess || at.type == cudaMemoryTypeUnregistered || at.devicePointer == nullptr) {
            (void)cudaGetLastError();
            return fail(LBM_ERR_INVALID_ARGUMENT,
                        "lbm_step_moments_to writes device memory or pinned host memory "
                        "(cudaHostAlloc / cudaHostRegister); this pointer is neither");
        }
        out[m] = static_cast<float*>(at.devicePointer);
    }
    // the previous readback into these (or other) buffers must have landed
    // before the host reads: lbm_readback_wait covers both kinds
    if (L->rb_pending) LBM_CUDA(cudaStreamWaitEvent(L->stream, L->rb_landed, 0));
    if (nsteps > 1)
        if (int rc = steps_impl(L, nsteps - 1, false)) return rc;
    if (int rc = lattice_readback_stream(L)) return rc;
    LBM_CUDA(launch_one_to(L, out));
    L->cur ^= 1;
    L->time += L->dt;
    L->steps += 1;
    L->mom_valid = false;
    LBM_CUDA(cudaEventRecord(L->rb_landed, L->stream));
    L->rb_pending = true;
    return LBM_OK;
}

int lbm_readback_wait(lbm_lattice* L) {
    if (int rc = check_handle(L)) return rc;
    if (!L->rb_pending) return LBM_OK;
    DeviceGuard g(L->dev);
    LBM_CUDA(cudaEventSynchronize(L->rb_landed));
    L->rb_pending = false;
    return LBM_OK;
}

int lbm_check(lbm_lattice* L, lbm_health* out) {
    if (int rc = check_handle(L)) return rc;
    if (!out) return fail(LBM_ERR_INVALID_ARGUMENT, "null health pointer");
    DeviceGuard g(L->dev);
    if (int rc = LBM_DISPATCH(L, health_t, L)) return rc;
    HealthPartial p;
    LBM_CUDA(cudaMemcpyAsync(&p, L->health + kHealthBlocks, sizeof(p), cudaMemcpyDeviceToHost,
                             L->stream));
    LBM_CUDA(cudaStreamSynchronize(L->stream));
    out->mass = p.mass;
    out->momentum_x = p.mx;
    out->momentum_y = p.my;
    out->min_population = p.minf;
    out->min_eq0 = p.mineq0;
    out->nonfinite_count = p.nonfinite;
    out->steps = L->steps;
    out->unstable = (p.mineq0 < 0.0 || p.nonfinite > 0) ? 1 : 0;
    out->reserved = 0;
    return LBM_OK;
}

int lbm_get_time(lbm_lattice* L, float* time, int64_t* steps) {
    if (int rc = check_handle(L)) return rc;
    if (time) *time = L->time;
    if (steps) *steps = L->steps;
    return LBM_OK;
}

int lbm_set_stream(lbm_lattice* L, void* stream) {
    if (int rc = check_handle(L)) return rc;
    DeviceGuard g(L->dev);
    LBM_CUDA(cudaStreamSynchronize(L->stream));
    L->stream = stream ? static_cast<cudaStream_t>(stream) : L->own;
    return LBM_OK;
}

int lbm_synchronize(lbm_lattice* L) {
    if (int rc = check_handle(L)) return rc;
    DeviceGuard g(L->dev);
    LBM_CUDA(cudaStreamSynchronize(L->stream));
    return LBM_OK;
}

int lbm_device_populations(lbm_lattice* L, void** base, int64_t* plane_stride, int* row_pitch) {
    if (int rc = check_handle(L)) return rc;
    if (base) *base = L->buf[L->cur];
    if (plane_stride) *plane_stride = L->plane;
    if (row_pitch) *row_pitch = L->pitch;
    return LBM_OK;
}

int lbm_set_tile(lbm_lattice* L, int cells_per_thread, int rows_per_block) {
    if (int rc = check_handle(L)) return rc;
    const int v = cells_per_thread ? cells_per_thread : default_cells(L->precision);
    const int r = rows_per_block ? rows_per_block : 4;
    if (!valid_cells(L->precision, v))
        return fail(LBM_ERR_INVALID_ARGUMENT, "cells_per_thread not available for this precision");
    if (r < 1 || r > 8 || (L->h + r - 1) / r > 65535 || 32 * r > 256)
        return fail(LBM_ERR_INVALID_ARGUMENT, "rows_per_block must be in [1, 8] and cover h");
    DeviceGuard g(L->dev);
    L->vcells = v; L->rows = r; L->dirty = true; ++L->version;
    if (int rc = refresh_tiles(L)) return rc;
    LBM_CUDA(cudaStreamSynchronize(L->stream));
    return LBM_OK;
}

// ---- checkpoint file ------------------------------------------------------
// Header (little-endian, 96 bytes) then the nine population planes in the
// lattice's storage type, row-major y * w + x (the C-ABI population layout;
// 16-bit storage keeps its raw deviation values, so a round trip is exact),
// then the solid mask (w * h bytes) when the lattice has one.
struct CheckpointHeader {
    char magic[8];            // "LBMSTATE"
    int32_t version;          // 1
    int32_t w, h, precision, flags, collision, has_solid, reserved0;
    float tau, tau_minus, dx, dt, fx, fy, time, reserved1;
    int64_t steps;
    int64_t reserved2[2];
};
static_assert(sizeof(CheckpointHeader) == 96, "checkpoint header layout");
constexpr char kStateMagic[8] = {'L', 'B', 'M', 'S', 'T', 'A', 'T', 'E'};

int lbm_save(lbm_lattice* L, const char* path) {
    if (int rc = check_handle(L)) return rc;
    if (!path) return fail(LBM_ERR_INVALID_ARGUMENT, "null path");
    DeviceGuard g(L->dev);
    CheckpointHeader hd{};
    std::memcpy(hd.magic, kStateMagic, 8);
    hd.version = 1;
    hd.w = L->w; hd.h = L->h; hd.precision = L->precision; hd.flags = L->flags;
    hd.collision = L->collision; hd.has_solid = L->has_solid ? 1 : 0;
    hd.tau = L->tau; hd.tau_minus = L->tau_minus; hd.dx = L->dx; hd.dt = L->dt;
    hd.fx = L->fx; hd.fy = L->fy; hd.time = L->time; hd.steps = L->steps;
    const size_t row = size_t(L->w) * L->esize, n = size_t(L->h) * row;
    std::vector<uint8_t> host(9 * n + (L->has_solid ? size_t(L->w) * L->h : 0));
    for (int i = 0; i < 9; ++i)
        LBM_CUDA(cudaMemcpy2DAsync(host.data() + i * n, row,
                                   static_cast<uint8_t*>(L->buf[L->cur]) + size_t(i) * L->plane * L->esize,
                                   size_t(L->pitch) * L->esize, row, L->h, cudaMemcpyDeviceToHost,
                                   L->stream));
    if (L->has_solid)
        LBM_CUDA(cudaMemcpy2DAsync(host.data() + 9 * n, L->w, L->solid, L->mpitch, L->w, L->h,
                                   cudaMemcpyDeviceToHost, L->stream));
    LBM_CUDA(cudaStreamSynchronize(L->stream));
    FILE* fp = std::fopen(path, "wb");
    if (!fp) return fail(LBM_ERR_INVALID_ARGUMENT, std::string("cannot open ") + path);
    const bool ok = std::fwrite(&hd, sizeof(hd), 1, fp) == 1 &&
                    std::fwrite(host.data(), 1, host.size(), fp) == host.size();
    if (std::fclose(fp) != 0 || !ok) return fail(LBM_ERR_INVALID_ARGUMENT, "checkpoint write failed");
    return LBM_OK;
}

int lbm_load(lbm_lattice* L, const char* path) {
    if (int rc = check_handle(L)) return rc;
    if (!path) return fail(LBM_ERR_INVALID_ARGUMENT, "null path");
    FILE* fp = std::fopen(path, "rb");
    if (!fp) return fail(LBM_ERR_INVALID_ARGUMENT, std::string("cannot open ") + path);
    CheckpointHeader hd{};
    bool ok = std::fread(&hd, sizeof(hd), 1, fp) == 1 && std::memcmp(hd.magic, kStateMagic, 8) == 0 &&
              hd.version == 1;
    if (ok && (hd.w != L->w || hd.h != L->h || hd.precision != L->precision ||
               (hd.flags & ~(LBM_FAST | LBM_ROUND_NEAREST)) != (L->flags & ~(LBM_FAST | LBM_ROUND_NEAREST)))) {
        std::fclose(fp);
        return fail(LBM_ERR_INVALID_ARGUMENT,
                    "checkpoint size, precision or boundary flags differ from the lattice's");
    }
    const size_t row = size_t(L->w) * L->esize, n = size_t(L->h) * row;
    std::vector<uint8_t> host;
    if (ok) {
        host.resize(9 * n + (hd.has_solid ? size_t(L->w) * L->h : 0));
        ok = std::fread(host.data(), 1, host.size(), fp) == host.size();
    }
    std::fclose(fp);
    if (!ok) return fail(LBM_ERR_INVALID_ARGUMENT, "not a lattice checkpoint (or truncated)");
    // Every header value is checked before the lattice changes, so a file
    // that fails leaves the lattice as it was.
    const bool trt = hd.collision == LBM_COLLISION_TRT;
    if (!(hd.dx > 0.f) || !(hd.dt > 0.f) || !std::isfinite(hd.dx) || !std::isfinite(hd.dt) ||
        (hd.collision != LBM_COLLISION_BGK && !trt) || !(hd.tau > 0.f) || !std::isfinite(hd.tau) ||
        (trt && (!(hd.tau_minus > 0.f) || !std::isfinite(hd.tau_minus))) ||
        !std::isfinite(hd.fx) || !std::isfinite(hd.fy) || !std::isfinite(hd.time) || hd.steps < 0)
        return fail(LBM_ERR_INVALID_ARGUMENT,
                    "checkpoint header holds an invalid discretization, collision, force, time or "
                    "step count; the lattice is unchanged");
    DeviceGuard g(L->dev);
    // The geometry upload is the one step that can still fail (device
    // memory); it goes first, and the setters below cannot fail.
    if (int rc = lbm_set_geometry(L, hd.has_solid ? host.data() + 9 * n : nullptr)) return rc;
    (void)lbm_set_discretization(L, hd.dx, hd.dt);
    (void)lbm_set_collision(L, hd.collision, hd.tau, hd.tau_minus);
    (void)lbm_set_force(L, hd.fx, hd.fy);
    for (int i = 0; i < 9; ++i)
        LBM_CUDA(cudaMemcpy2DAsync(static_cast<uint8_t*>(L->buf[L->cur]) + size_t(i) * L->plane * L->esize,
                                   size_t(L->pitch) * L->esize, host.data() + i * n, row, row, L->h,
                                   cudaMemcpyHostToDevice, L->stream));
    LBM_CUDA(cudaStreamSynchronize(L->stream));
    L->flags = (L->flags & ~(LBM_FAST | LBM_ROUND_NEAREST)) | (hd.flags & (LBM_FAST | LBM_ROUND_NEAREST));
    L->time = hd.time;
    L->steps = hd.steps;
    L->mom_valid = false;
    L->dirty = true;
    ++L->version;
    return LBM_OK;
}

}  // extern "C"
