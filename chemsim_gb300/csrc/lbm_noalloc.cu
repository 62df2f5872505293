// lbm_noalloc.cu — health check of caller-owned device populations that
// allocates no device memory.
//
// Who needs it: callers that must not call cudaMalloc.  A renderer or game
// loop that hands the lattice to a frame callback cannot afford the implicit
// device synchronisation of cudaMalloc/cudaFree; a host application that has
// reserved the whole device for its own memory pool has nothing left for a
// library to allocate; and a plugin host may forbid libraries from allocating
// at all.  lbm_check needs an lbm_lattice handle, whose creation allocates;
// lbm_check_device_noalloc needs only a pointer to populations the caller
// already owns (for example those lbm_device_populations returns).
//
// The reduction's scratch (one partial per block plus the result) lives in the
// file-scope device array g_noalloc_scratch below: 16385 partials of 48 bytes
// (768 KiB), held by every GPU that loads this library until the process
// exits.  One block reduces kNoAllocCellsPerBlock cells, so the largest
// lattice is kNoAllocMaxBlocks * kNoAllocCellsPerBlock = 2^28 cells
// (16384 x 16384); larger lattices are rejected.
#include <cuda.h>

#include <cmath>
#include <mutex>
#include <string>

#include "lbm_aux.cuh"

using namespace lbmk;

namespace {

constexpr int kNoAllocMaxBlocks = 16384;
constexpr int64_t kNoAllocCellsPerBlock = 16384;
constexpr int kNoAllocSlots = 64;

// Partials [0, kNoAllocMaxBlocks) and the result at index kNoAllocMaxBlocks.
static __device__ __align__(256) HealthPartial g_noalloc_scratch[kNoAllocMaxBlocks + 1];

// Device address of g_noalloc_scratch, resolved once per CUDA context and
// kept under the context's ID.  A context ID is never reused within a
// process, so a context that replaces another (the new primary context after
// cudaDeviceReset, whose module copy may sit elsewhere) or a second context
// on the same device never finds another context's address.
struct ScratchSlot {
    unsigned long long ctx_id;
    HealthPartial* ptr;
};
std::mutex g_noalloc_mutex;
ScratchSlot g_noalloc_slots[kNoAllocSlots] = {};
int g_noalloc_next = 0;

using CtxGetCurrentFn = CUresult (*)(CUcontext*);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long*);

// ID of the calling thread's current context (0 when none is current or the
// driver entry points are unavailable; the address is then resolved afresh).
unsigned long long current_ctx_id() {
    static CtxGetCurrentFn get_current = nullptr;
    static CtxGetIdFn get_id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) ==
                cudaSuccess && q == cudaDriverEntryPointSuccess)
            get_current = reinterpret_cast<CtxGetCurrentFn>(f);
        f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) ==
                cudaSuccess && q == cudaDriverEntryPointSuccess)
            get_id = reinterpret_cast<CtxGetIdFn>(f);
        (void)cudaGetLastError();
    });
    if (!get_current || !get_id) return 0;
    CUcontext ctx = nullptr;
    unsigned long long id = 0;
    if (get_current(&ctx) != CUDA_SUCCESS || ctx == nullptr || get_id(ctx, &id) != CUDA_SUCCESS)
        return 0;
    return id;
}


// Final reduction of the partials by one block of 256 threads: thread t sums
// partials t, t + 256, ...; the 256 results are combined in a fixed order, so
// the result is deterministic.
__global__ void __launch_bounds__(256)
noalloc_final_kernel(const HealthPartial* __restrict__ partial, int nblocks,
                     HealthPartial* __restrict__ out) {
    __shared__ HealthPartial s[256];
    HealthPartial p{0.0, 0.0, 0.0, INFINITY, INFINITY, 0};
    for (int k = threadIdx.x; k < nblocks; k += blockDim.x) {
        p.mass += partial[k].mass;
        p.mx += partial[k].mx;
        p.my += partial[k].my;
        p.minf = fmin(p.minf, partial[k].minf);
        p.mineq0 = fmin(p.mineq0, partial[k].mineq0);
        p.nonfinite += partial[k].nonfinite;
    }
    s[threadIdx.x] = p;
    __syncthreads();
    if (threadIdx.x == 0) {
        HealthPartial r{0.0, 0.0, 0.0, INFINITY, INFINITY, 0};
        for (int k = 0; k < int(blockDim.x); ++k) {
            r.mass += s[k].mass;
            r.mx += s[k].mx;
            r.my += s[k].my;
            r.minf = fmin(r.minf, s[k].minf);
            r.mineq0 = fmin(r.mineq0, s[k].mineq0);
            r.nonfinite += s[k].nonfinite;
        }
        *out = r;
    }
}

template <class S>
cudaError_t noalloc_launch(const void* f, int w, int h, int pitch, int64_t plane,
                           const Consts<typename Store<S>::CT>& c, int nblocks,
                           HealthPartial* scratch, cudaStream_t stream) {
    health_kernel<S><<<nblocks, 256, 0, stream>>>(static_cast<const S*>(f), w, h, pitch, plane, c,
                                                  scratch);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    noalloc_final_kernel<<<1, 256, 0, stream>>>(scratch, nblocks, scratch + kNoAllocMaxBlocks);
    return cudaGetLastError();
}

// Errors are reported through lbm_last_error_string, like every entry point.
int noalloc_fail(int code, const std::string& msg) {
    lbmk::set_last_error(msg);
    return code;
}

template <class CT>
Consts<CT> noalloc_consts(int precision, float dx, float dt) {
    // The constants of the health reduction: weights and 1/cs^2 terms
    // (src/lbm.rs:43-71, 83-85), the deviation-storage scale.
    Consts<CT> c{};
    const CT n[9] = {CT(16), CT(4), CT(4), CT(4), CT(4), CT(1), CT(1), CT(1), CT(1)};
    for (int i = 0; i < 9; ++i) c.wt[i] = n[i] / CT(36);
    const CT cs = CT(dx) / (CT(std::sqrt(CT(3))) * CT(dt));
    const CT cs2 = cs * cs;
    const CT cs4 = cs2 * cs2;
    c.k1 = CT(1) / cs2;
    c.k2 = CT(1) / (CT(2) * cs4);
    c.k3 = CT(-1) / (CT(2) * cs2);
    if (precision == LBM_F16DEV) { c.dscale = CT(kHalfDevScale); c.dinv = CT(1) / CT(kHalfDevScale); }
    else if (precision == LBM_BF16DEV) { c.dscale = CT(kBf16DevScale); c.dinv = CT(1) / CT(kBf16DevScale); }
    else { c.dscale = CT(1); c.dinv = CT(1); }
    return c;
}

}  // namespace

extern "C" {

int lbm_check_device_noalloc(const void* populations, int precision, int w, int h,
                             int row_pitch, int64_t plane_stride, float delta_x,
                             float delta_t, void* stream, lbm_health* out) {
    if (!populations || !out)
        return noalloc_fail(LBM_ERR_INVALID_ARGUMENT, "populations and out must not be null");
    if (precision < LBM_F32 || precision > LBM_BF16DEV)
        return noalloc_fail(LBM_ERR_INVALID_ARGUMENT, "unknown precision");
    if (w < 1 || h < 1 || row_pitch < w || plane_stride < int64_t(row_pitch) * h)
        return noalloc_fail(LBM_ERR_INVALID_ARGUMENT,
                            "need w, h >= 1, row_pitch >= w and plane_stride >= row_pitch * h");
    if (!(delta_x > 0.f) || !(delta_t > 0.f))
        return noalloc_fail(LBM_ERR_INVALID_ARGUMENT, "delta_x and delta_t must be > 0");
    const int64_t cells = int64_t(w) * h;
    if (cells > int64_t(kNoAllocMaxBlocks) * kNoAllocCellsPerBlock)
        return noalloc_fail(LBM_ERR_INVALID_ARGUMENT,
                            "lattice too large for lbm_check_device_noalloc: at most 268435456 "
                            "cells (16384 x 16384); use lbm_check");
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return noalloc_fail(LBM_ERR_CUDA, cudaGetErrorString(e));
    HealthPartial* scratch = nullptr;
    {
        // Set-up, once per context, with the device current: the host-side
        // name g_noalloc_scratch is not a device address; ask the runtime.
        // Before the runtime's first call on this thread no context may be
        // current (ID 0); cudaGetSymbolAddress then makes the device's
        // primary context current, and its ID is read afterwards.
        unsigned long long id = current_ctx_id();
        std::lock_guard<std::mutex> lock(g_noalloc_mutex);
        for (const ScratchSlot& slot : g_noalloc_slots)
            if (id != 0 && slot.ctx_id == id) scratch = slot.ptr;
        if (!scratch) {
            void* p = nullptr;
            e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (e != cudaSuccess) {
                (void)cudaGetLastError();
                return noalloc_fail(LBM_ERR_CUDA,
                                    std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
            }
            scratch = static_cast<HealthPartial*>(p);
            if (id == 0) id = current_ctx_id();
            if (id != 0) {
                g_noalloc_slots[g_noalloc_next] = ScratchSlot{id, scratch};
                g_noalloc_next = (g_noalloc_next + 1) % kNoAllocSlots;
            }
        }
    }
    const int nblocks = int((cells + kNoAllocCellsPerBlock - 1) / kNoAllocCellsPerBlock);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    (void)cudaGetLastError();
    switch (precision) {
        case LBM_F32:
            e = noalloc_launch<float>(populations, w, h, row_pitch, plane_stride,
                                      noalloc_consts<float>(precision, delta_x, delta_t), nblocks,
                                      scratch, s);
            break;
        case LBM_F64:
            e = noalloc_launch<double>(populations, w, h, row_pitch, plane_stride,
                                       noalloc_consts<double>(precision, delta_x, delta_t), nblocks,
                                       scratch, s);
            break;
        case LBM_F16DEV:
            e = noalloc_launch<__half>(populations, w, h, row_pitch, plane_stride,
                                       noalloc_consts<float>(precision, delta_x, delta_t), nblocks,
                                       scratch, s);
            break;
        default:
            e = noalloc_launch<__nv_bfloat16>(populations, w, h, row_pitch, plane_stride,
                                              noalloc_consts<float>(precision, delta_x, delta_t),
                                              nblocks, scratch, s);
            break;
    }
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        return noalloc_fail(LBM_ERR_CUDA, std::string("health kernels: ") + cudaGetErrorString(e));
    }
    HealthPartial r;
    e = cudaMemcpyAsync(&r, scratch + kNoAllocMaxBlocks, sizeof(r), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        return noalloc_fail(LBM_ERR_CUDA, std::string("result copy: ") + cudaGetErrorString(e));
    }
    out->mass = r.mass;
    out->momentum_x = r.mx;
    out->momentum_y = r.my;
    out->min_population = r.minf;
    out->min_eq0 = r.mineq0;
    out->nonfinite_count = r.nonfinite;
    out->steps = 0;
    out->unstable = (r.mineq0 < 0.0 || r.nonfinite > 0) ? 1 : 0;
    out->reserved = 0;
    return LBM_OK;
}

}  // extern "C"
