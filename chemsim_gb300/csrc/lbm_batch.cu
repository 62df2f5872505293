// lbm_batch.cu — many independent lattices advanced together.
//
// A batch owns n ordinary lattices (lbm_lattice handles, so every
// single-lattice entry point works on a member) and advances all of them by
// one launch per time step.  The launch covers a list of work items, one per
// warp: (member, row, warp tile) of every member, general items first, then
// each member in blocks of 4 rows of one tile column, so the 4 warps of a CTA
// share the rows they pull from.  Each warp runs the same interior / general /
// link-mask step code as a single lattice, so a member's results do not depend
// on whether it was stepped alone or in a batch.  Runs of steps replay a
// captured CUDA graph.  The autotuner picks the batch's tile width (2 or 4
// cells per thread, one kernel each).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "lbm_handle.cuh"

using namespace lbmk;

struct lbm_batch_member_dev {
    StepArgs<float> a;      // the member's step arguments at build time (both parities
                            // share everything but src / dst, which the items carry)
};

// One warp's work item, 32 bytes: everything a warp needs to issue its
// population loads, so no dependent read precedes them.
struct BatchItem {
    const float* buf0;      // the member's buffer that is the source at parity 0
    const float* buf1;      // the other buffer
    uint32_t member_kind;   // member index | kind << 24
    uint32_t row_tile;      // row << 12 | warp tile
    uint32_t w_pitch;       // w | (row pitch / 32) << 18
    uint32_t h;
};
static_assert(sizeof(BatchItem) == 32, "32-byte items");

struct lbm_batch {
    std::vector<lbm_lattice*> members;
    std::vector<uint64_t> built_version;
    std::vector<int> built_cur;
    lbm_batch_member_dev* d_members = nullptr;
    BatchItem* d_tasks = nullptr;     // work items
    int ntasks = 0;
    size_t tasks_cap = 0;
    int par = 0;                      // steps since the table was built, mod 2
    bool built = false;
    int frame = 0, fast = 1;
    int V = 4;                        // cells per thread of every member in batch steps
    int resident[2] = {0, 0};         // resident warps of the V = 2 and V = 4 kernels, whole GPU
    cudaStream_t own = nullptr, stream = nullptr;
    cudaGraphExec_t graph[2] = {nullptr, nullptr};
    int dev = 0;
    bool owns = true;                 // destroys its members (false: a tuning view)
};

namespace {

#ifndef LBM_BATCH_WARPS
#define LBM_BATCH_WARPS 4
#endif
constexpr int kTaskWarps = LBM_BATCH_WARPS;
constexpr int kBatchGraphSteps = 16;
constexpr int kDefaultV = 4;

// Item kinds (bits 24-31 of the item's first word).
enum : uint32_t { kGeneral = 0, kWrap = 1, kInterior = 2, kLinks = 3 };

#ifndef LBM_BATCH_PREFETCH
#define LBM_BATCH_PREFETCH 1
#endif
// Prefetch distance in percent of the resident warps (one wave: 100).
#ifndef LBM_BATCH_PF_PCT
#define LBM_BATCH_PF_PCT 130
#endif

// A batch item's step arguments in the shape the step code reads: the
// addressing fields come from the item; the member's other arguments
// (collision constants, flags, mask, link masks) are read from the member
// table where a path uses them, after the population loads are issued.
// Moment outputs and the single-lattice prefetch are compiled out.
struct BatchView {
    const void* src;
    void* dst;
    int64_t plane;
    int pitch, w, h;
    const Consts<float>& c;
    const int& flags;
    const uint8_t* const& solid;
    const int& mpitch;
    const int& ntiles;
    const uint4* const& links;
    static constexpr float* mom_rho = nullptr;
    static constexpr float* mom_ux = nullptr;
    static constexpr float* mom_uy = nullptr;
    static constexpr int mom_pitch = 0;
    static constexpr int pf_rows = 0;
    __device__ __forceinline__ BatchView(const BatchItem& it, const StepArgs<float>& m, int parity)
        : src(parity ? it.buf1 : it.buf0),
          dst(const_cast<float*>(parity ? it.buf0 : it.buf1)),
          plane(int64_t((it.w_pitch >> 18) * 32u) * it.h),
          pitch(int((it.w_pitch >> 18) * 32u)),
          w(int(it.w_pitch & 0x3ffffu)),
          h(int(it.h)),
          c(m.c), flags(m.flags), solid(m.solid), mpitch(m.mpitch), ntiles(m.ntiles), links(m.links) {}
};

// L2 prefetch of the rows item q pulls, one plane a lane (the range is
// clipped to the row's pitch, so it stays inside the member's buffer).
template <int V, int FRAME>
__device__ __forceinline__ void prefetch_item(const BatchItem* __restrict__ items, int nitems, int q,
                                              int parity, int lane) {
    if (!LBM_BATCH_PREFETCH || lane >= 9 || q >= nitems) return;
    const BatchItem next = items[q];
    const int h = int(next.h), pitch = int((next.w_pitch >> 18) * 32u);
    const int ys = int(next.row_tile >> 12) - DROW(FRAME, lane);
    const int x0 = int(next.row_tile & 4095u) * 32 * V;
    if (ys >= 0 && ys < h) {
        const int n = min(32 * V, pitch - x0);
        const float* p = (parity ? next.buf1 : next.buf0) + lane * (int64_t(pitch) * h) +
                         int64_t(ys) * pitch + x0;
        asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" :: "l"(p), "r"(n * 4) : "memory");
    }
}

// One warp = one work item: the kind dispatch is warp-uniform.  After its own
// item the warp prefetches into L2 the rows of the item about 1.3 waves of
// resident warps ahead.
template <int V, int FRAME, bool FAST>
__device__ __forceinline__ void batch_item(const lbm_batch_member_dev* __restrict__ members,
                                           const BatchItem* __restrict__ items, int nitems, int parity,
                                           int pf) {
    const int lane = threadIdx.x;
    const int it = blockIdx.x * blockDim.y + threadIdx.y;
    if (it >= nitems) return;
    const BatchItem item = items[it];
    const BatchView a(item, members[item.member_kind & 0xffffffu].a, parity);
    const int y = int(item.row_tile >> 12), tile = int(item.row_tile & 4095u);
    const int x0 = (tile * 32 + lane) * V;
    switch (item.member_kind >> 24) {      // warp-uniform
        case kGeneral: step_general<float, V, FRAME, FAST>(a, y, tile, lane); break;
        case kWrap: step_interior_wrap<float, V, FRAME, FAST>(a, y, x0, lane); break;
        case kInterior: step_interior<float, V, FRAME, FAST>(a, y, x0, lane); break;
        default: step_interior<float, V, FRAME, FAST, false, true>(a, y, x0, lane, tile); break;
    }
    prefetch_item<V, FRAME>(items, nitems, it + pf, parity, lane);
}

// Registers, CTAs of 4 warps: 4 cells per thread capped at 96 (5 CTAs per
// SM), 2 cells at 64 (8 CTAs); the general path spills a little at both.
// 512-member mix, one GB300, fraction of the copy bandwidth at 4 cells per
// thread: CTAs of 8 warps at 80 registers 0.765, of 4 warps at 80 0.775, of
// 4 warps at 96 0.784.
#ifndef LBM_BATCH_V4_MAXNREG
#define LBM_BATCH_V4_MAXNREG 96
#endif
template <int FRAME, bool FAST>
__global__ void __maxnreg__(LBM_BATCH_V4_MAXNREG)
lbm_batch_kernel_v4(const lbm_batch_member_dev* __restrict__ members, const BatchItem* __restrict__ items,
                    int nitems, int parity, int pf) {
    batch_item<4, FRAME, FAST>(members, items, nitems, parity, pf);
}
#ifdef LBM_BATCH_V2_MAXNREG
template <int FRAME, bool FAST>
__global__ void __maxnreg__(LBM_BATCH_V2_MAXNREG)
#else
template <int FRAME, bool FAST>
__global__ void __launch_bounds__(256, 4)
#endif
lbm_batch_kernel_v2(const lbm_batch_member_dev* __restrict__ members, const BatchItem* __restrict__ items,
                    int nitems, int parity, int pf) {
    batch_item<2, FRAME, FAST>(members, items, nitems, parity, pf);
}

using BatchKernel = void (*)(const lbm_batch_member_dev*, const BatchItem*, int, int, int);

BatchKernel pick_kernel(int V, int frame, int fast) {
    if (V == 2) {
        if (frame) return fast ? lbm_batch_kernel_v2<1, true> : lbm_batch_kernel_v2<1, false>;
        return fast ? lbm_batch_kernel_v2<0, true> : lbm_batch_kernel_v2<0, false>;
    }
    if (frame) return fast ? lbm_batch_kernel_v4<1, true> : lbm_batch_kernel_v4<1, false>;
    return fast ? lbm_batch_kernel_v4<0, true> : lbm_batch_kernel_v4<0, false>;
}

int bfail(int code, const std::string& msg) { return lattice_fail(code, msg); }

#define BATCH_CUDA(expr)                                                             \
    do {                                                                             \
        cudaError_t e__ = (expr);                                                    \
        if (e__ != cudaSuccess) {                                                    \
            (void)cudaGetLastError();                                                \
            return bfail(e__ == cudaErrorMemoryAllocation ? LBM_ERR_OUT_OF_MEMORY     \
                                                          : LBM_ERR_CUDA,            \
                         std::string(#expr) + ": " + cudaGetErrorString(e__));       \
        }                                                                            \
    } while (0)

void drop_graphs(lbm_batch* B) {
    for (auto& g : B->graph) {
        if (g) cudaGraphExecDestroy(g);
        g = nullptr;
    }
}

// (Re)builds the device member table and the item list when a member changed.
// Members step at the batch's tile width: a member set to another width (by
// lbm_set_tile) is set back to it here.
int ensure_table(lbm_batch* B) {
    const int n = int(B->members.size());
    for (lbm_lattice* L : B->members)
        if (L->vcells != B->V)
            if (int rc = lbm_set_tile(L, B->V, L->rows)) return rc;
    bool changed = !B->built;
    for (int i = 0; i < n && !changed; ++i) {
        const lbm_lattice* L = B->members[i];
        if (L->version != B->built_version[i] || L->cur != (B->built_cur[i] ^ B->par)) changed = true;
    }
    if (!changed) return LBM_OK;
    std::vector<lbm_batch_member_dev> host(n);
    std::vector<BatchItem> general, rest;
    std::vector<uint8_t> flags;
    for (int i = 0; i < n; ++i) {
        lbm_lattice* L = B->members[i];
        host[i].a = lattice_args<float>(L, L->cur, false);
        if (L->pitch % 32 != 0 || L->pitch / 32 >= (1 << 14) || L->w >= (1 << 18) ||
            L->plane != int64_t(L->pitch) * L->h)
            return bfail(LBM_ERR_INVALID_ARGUMENT, "batch member row pitch or width out of range");
        const float* buf0 = static_cast<const float*>(L->buf[L->cur]);
        const float* buf1 = static_cast<const float*>(L->buf[L->cur ^ 1]);
        const uint32_t w_pitch = uint32_t(L->w) | (uint32_t(L->pitch / 32) << 18);
        B->built_version[i] = L->version;
        B->built_cur[i] = L->cur;
        flags.resize(size_t(L->h) * L->ntiles);
        BATCH_CUDA(cudaMemcpyAsync(flags.data(), L->tflags, flags.size(), cudaMemcpyDeviceToHost,
                                   B->stream));
        BATCH_CUDA(cudaStreamSynchronize(B->stream));
        for (int r0 = 0; r0 < L->h; r0 += kTaskWarps)
            for (int t = 0; t < L->ntiles; ++t)
                for (int r = r0; r < std::min(L->h, r0 + kTaskWarps); ++r) {
                    const uint8_t fl = flags[size_t(r) * L->ntiles + t];
                    // flag 3 (solids nearby, no lattice edge in reach) runs the
                    // interior code with link masks when the member has them
                    const uint32_t kind = fl == 0 ? kInterior : fl == 2 ? kWrap
                                        : (fl == 3 && L->use_links) ? kLinks : kGeneral;
                    const BatchItem item{buf0, buf1, uint32_t(i) | (kind << 24),
                                         (uint32_t(r) << 12) | uint32_t(t), w_pitch, uint32_t(L->h)};
                    (kind == kGeneral ? general : rest).push_back(item);
                }
    }
    // general items first: their longer latency overlaps the rest
    std::vector<BatchItem> tasks(general);
    tasks.insert(tasks.end(), rest.begin(), rest.end());
    if (!B->d_members) BATCH_CUDA(cudaMalloc(&B->d_members, sizeof(lbm_batch_member_dev) * n));
    BATCH_CUDA(cudaMemcpyAsync(B->d_members, host.data(), sizeof(lbm_batch_member_dev) * n,
                               cudaMemcpyHostToDevice, B->stream));
    if (tasks.size() > B->tasks_cap) {
        if (B->d_tasks) cudaFree(B->d_tasks);
        B->d_tasks = nullptr;
        B->tasks_cap = 0;
        BATCH_CUDA(cudaMalloc(&B->d_tasks, sizeof(BatchItem) * tasks.size()));
        B->tasks_cap = tasks.size();
    }
    if (!tasks.empty())
        BATCH_CUDA(cudaMemcpyAsync(B->d_tasks, tasks.data(), sizeof(BatchItem) * tasks.size(),
                                   cudaMemcpyHostToDevice, B->stream));
    BATCH_CUDA(cudaStreamSynchronize(B->stream));
    B->ntasks = int(tasks.size());
    B->par = 0;
    B->built = true;
    drop_graphs(B);
    return LBM_OK;
}

// One step: one launch, one warp per item.
cudaError_t launch(lbm_batch* B, int parity) {
    if (B->ntasks == 0) return cudaSuccess;
    const int grid = (B->ntasks + kTaskWarps - 1) / kTaskWarps;
    const int pf = std::max(1, int(int64_t(B->resident[B->V == 4]) * LBM_BATCH_PF_PCT / 100));
    pick_kernel(B->V, B->frame, B->fast)<<<grid, dim3(32, kTaskWarps), 0, B->stream>>>(
        B->d_members, B->d_tasks, B->ntasks, parity, pf);
    return cudaGetLastError();
}

int ensure_graph(lbm_batch* B) {
    const int p = B->par & 1;
    if (B->graph[p]) return LBM_OK;
    BATCH_CUDA(cudaStreamBeginCapture(B->stream, cudaStreamCaptureModeThreadLocal));
    cudaError_t err = cudaSuccess;
    for (int s = 0; s < kBatchGraphSteps && err == cudaSuccess; ++s) err = launch(B, (p + s) & 1);
    cudaGraph_t g = nullptr;
    cudaError_t e2 = cudaStreamEndCapture(B->stream, &g);
    if (err != cudaSuccess || e2 != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        (void)cudaGetLastError();
        return bfail(LBM_ERR_CUDA, std::string("batch capture: ") +
                                       cudaGetErrorString(err != cudaSuccess ? err : e2));
    }
    cudaError_t e3 = cudaGraphInstantiate(&B->graph[p], g, 0);
    cudaGraphDestroy(g);
    if (e3 != cudaSuccess) {
        B->graph[p] = nullptr;
        (void)cudaGetLastError();
        return bfail(LBM_ERR_CUDA, std::string("batch graph: ") + cudaGetErrorString(e3));
    }
    return LBM_OK;
}

int width_class(int w) {
    if (w <= 96) return 0;
    if (w <= 192) return 1;
    if (w <= 384) return 2;
    if (w <= 768) return 3;
    return 4;
}

// Candidate tile widths (cells per thread; the batch kernel's warp tile is
// 32 x that wide), one kernel each.
const int kCandidates[2] = {2, 4};

}  // namespace

extern "C" {

int lbm_batch_create(int n, const lbm_desc* descs, int flags, lbm_batch** out) {
    if (!out) return bfail(LBM_ERR_INVALID_ARGUMENT, "out must not be null");
    *out = nullptr;
    if (n < 1 || n > (1 << 24) || !descs)
        return bfail(LBM_ERR_INVALID_ARGUMENT, "need 1 <= n <= 16777216 lattice descriptions");
    if (flags & ~(LBM_FRAME_XY | LBM_FAST))
        return bfail(LBM_ERR_INVALID_ARGUMENT, "batch flags may only hold LBM_FRAME_XY and LBM_FAST");
    lbm_batch* B = new lbm_batch();
    B->frame = (flags & LBM_FRAME_XY) ? 1 : 0;
    B->fast = (flags & LBM_FAST) ? 1 : 0;
    B->V = kDefaultV;
    auto cleanup = [&](int rc) { lbm_batch_destroy(B); return rc; };
    if (cudaGetDevice(&B->dev) != cudaSuccess) return cleanup(bfail(LBM_ERR_CUDA, "no device"));
    for (int i = 0; i < n; ++i) {
        const lbm_desc& d = descs[i];
        if (d.flags & (LBM_FRAME_XY | LBM_FAST))
            return cleanup(bfail(LBM_ERR_INVALID_ARGUMENT,
                                 "member flags carry boundaries only; frame and arithmetic are the batch's"));
        lbm_lattice* L = nullptr;
        int rc = lbm_create(d.w, d.h, d.tau, LBM_F32, d.flags | flags, &L);
        if (rc) return cleanup(rc);
        B->members.push_back(L);
        B->built_version.push_back(~uint64_t(0));
        B->built_cur.push_back(0);
        if (d.fx != 0.f || d.fy != 0.f) {
            if ((rc = lbm_set_force(L, d.fx, d.fy))) return cleanup(rc);
        }
        if (d.solid) {
            if ((rc = lbm_set_geometry(L, d.solid))) return cleanup(rc);
        }
    }
    cudaError_t e = cudaStreamCreateWithFlags(&B->own, cudaStreamNonBlocking);
    if (e != cudaSuccess) return cleanup(bfail(LBM_ERR_CUDA, cudaGetErrorString(e)));
    B->stream = B->own;
    // Members run on the batch's stream, so their own calls are ordered after
    // batch steps without any host synchronisation.
    for (lbm_lattice* L : B->members)
        if (int rc = lbm_set_stream(L, B->stream)) return cleanup(rc);
    // Resident warps of each kernel on the whole GPU: the prefetch distance.
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, B->dev);
    for (int q = 0; q < 2; ++q) {
        int per_sm = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, pick_kernel(2 + 2 * q, B->frame, B->fast),
                                                      32 * kTaskWarps, 0);
        B->resident[q] = std::max(1, sms) * std::max(1, per_sm) * kTaskWarps;
    }
    *out = B;
    return LBM_OK;
}

int lbm_batch_destroy(lbm_batch* B) {
    if (!B) return LBM_OK;
    if (B->stream) cudaStreamSynchronize(B->stream);
    drop_graphs(B);
    if (B->owns)
        for (lbm_lattice* L : B->members) lbm_destroy(L);
    if (B->d_members) cudaFree(B->d_members);
    if (B->d_tasks) cudaFree(B->d_tasks);
    if (B->own) cudaStreamDestroy(B->own);
    delete B;
    return LBM_OK;
}

int lbm_batch_size(lbm_batch* B, int* n) {
    if (!B || !n) return bfail(LBM_ERR_INVALID_ARGUMENT, "null argument");
    *n = int(B->members.size());
    return LBM_OK;
}

int lbm_batch_lattice(lbm_batch* B, int index, lbm_lattice** out) {
    if (!B || !out) return bfail(LBM_ERR_INVALID_ARGUMENT, "null argument");
    if (index < 0 || index >= int(B->members.size()))
        return bfail(LBM_ERR_INVALID_ARGUMENT, "member index out of range");
    *out = B->members[index];
    return LBM_OK;
}

int lbm_batch_step(lbm_batch* B, int nsteps) {
    if (!B) return bfail(LBM_ERR_INVALID_ARGUMENT, "null batch");
    if (nsteps < 0) return bfail(LBM_ERR_INVALID_ARGUMENT, "nsteps must be >= 0");
    if (nsteps == 0) return LBM_OK;
    if (int rc = ensure_table(B)) return rc;
    int left = nsteps;
    if (left >= kBatchGraphSteps) {
        if (int rc = ensure_graph(B)) return rc;
        while (left >= kBatchGraphSteps) {
            BATCH_CUDA(cudaGraphLaunch(B->graph[B->par & 1], B->stream));
            left -= kBatchGraphSteps;     // an even count: parity unchanged
        }
    }
    for (; left > 0; --left) {
        BATCH_CUDA(launch(B, B->par & 1));
        B->par ^= 1;
    }
    for (lbm_lattice* L : B->members) lattice_advance(L, nsteps);
    return LBM_OK;
}

int lbm_batch_synchronize(lbm_batch* B) {
    if (!B) return bfail(LBM_ERR_INVALID_ARGUMENT, "null batch");
    BATCH_CUDA(cudaStreamSynchronize(B->stream));
    return LBM_OK;
}

int lbm_batch_set_stream(lbm_batch* B, void* stream) {
    if (!B) return bfail(LBM_ERR_INVALID_ARGUMENT, "null batch");
    BATCH_CUDA(cudaStreamSynchronize(B->stream));
    B->stream = stream ? static_cast<cudaStream_t>(stream) : B->own;
    for (lbm_lattice* L : B->members)
        if (int rc = lbm_set_stream(L, B->stream)) return rc;
    return LBM_OK;
}

int lbm_batch_set_tile(lbm_batch* B, int cells_per_thread) {
    if (!B) return bfail(LBM_ERR_INVALID_ARGUMENT, "null batch");
    if (cells_per_thread != 2 && cells_per_thread != 4)
        return bfail(LBM_ERR_INVALID_ARGUMENT, "a batch steps with 2 or 4 cells per thread");
    BATCH_CUDA(cudaStreamSynchronize(B->stream));
    B->V = cells_per_thread;
    return ensure_table(B);
}

int lbm_batch_tile(lbm_batch* B, int* cells_per_thread) {
    if (!B || !cells_per_thread) return bfail(LBM_ERR_INVALID_ARGUMENT, "null argument");
    *cells_per_thread = B->V;
    return LBM_OK;
}

int lbm_batch_autotune(lbm_batch* B, const char* cache_path, int steps_per_trial) {
    if (!B) return bfail(LBM_ERR_INVALID_ARGUMENT, "null batch");
    if (steps_per_trial <= 0) steps_per_trial = 24;
    cudaDeviceProp prop;
    BATCH_CUDA(cudaGetDeviceProperties(&prop, B->dev));
    char keybuf[320];
    std::snprintf(keybuf, sizeof(keybuf), "%s|f32|%s|%s", prop.name, B->frame ? "xy" : "ref",
                  B->fast ? "fast" : "strict");
    const std::string key(keybuf);
    // Cache: one JSON object per line, {"key": "...", "V": v, ...}; a line of
    // this key gives the choice, lines of other keys are kept.
    std::vector<std::string> kept;
    int cached = 0;
    if (cache_path) {
        if (FILE* fh = std::fopen(cache_path, "r")) {
            char line[1024];
            while (std::fgets(line, sizeof(line), fh)) {
                const char* k = std::strstr(line, "\"key\": \"");
                if (!k) continue;
                k += 8;
                const char* ke = std::strchr(k, '"');
                if (!ke) continue;
                const std::string lk(k, ke - k);
                const char* pv = std::strstr(line, "\"V\": ");
                const int v = pv ? std::atoi(pv + 5) : 0;
                std::string body(line);
                while (!body.empty() && (body.back() == '\n' || body.back() == ',' || body.back() == ' '))
                    body.pop_back();
                if (lk == key && (v == 2 || v == 4)) cached = v;
                else kept.push_back(body);
            }
            std::fclose(fh);
        }
    }
    if (cached) {
        B->V = cached;
        return ensure_table(B);
    }
    // Time both widths on each width class's members in turn, through a
    // non-owning view of them, with their state saved first and restored
    // afterwards (one class at a time bounds the saved copy), and sum.
    double total_ms[2] = {0.0, 0.0}, cells = 0.0;
    for (int c = 0; c < 5; ++c) {
        lbm_batch view;
        view.owns = false;
        view.frame = B->frame;
        view.fast = B->fast;
        std::copy(B->resident, B->resident + 2, view.resident);
        view.stream = B->stream;
        view.dev = B->dev;
        struct Saved { void* f; int cur; float time; int64_t steps; int v, rows; };
        std::vector<Saved> saved;
        int rc = LBM_OK;
        for (lbm_lattice* L : B->members) {
            if (width_class(L->w) != c) continue;
            Saved sv{nullptr, L->cur, L->time, L->steps, L->vcells, L->rows};
            const size_t bytes = size_t(9) * L->plane * L->esize;
            cudaError_t e = cudaMallocAsync(&sv.f, bytes, B->stream);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(sv.f, L->buf[L->cur], bytes, cudaMemcpyDeviceToDevice, B->stream);
            if (e != cudaSuccess) {
                if (sv.f) cudaFreeAsync(sv.f, B->stream);
                rc = bfail(LBM_ERR_CUDA, cudaGetErrorString(e));
                (void)cudaGetLastError();
                break;
            }
            saved.push_back(sv);
            view.members.push_back(L);
            view.built_version.push_back(~uint64_t(0));
            view.built_cur.push_back(0);
            cells += double(L->w) * L->h;
        }
        cudaEvent_t e0 = nullptr, e1 = nullptr;
        if (!rc && !view.members.empty()) { cudaEventCreate(&e0); cudaEventCreate(&e1); }
        for (int q = 0; q < 2 && !rc && !view.members.empty(); ++q) {
            view.V = kCandidates[q];
            view.built = false;
            drop_graphs(&view);
            rc = lbm_batch_step(&view, 4);
            if (rc) break;
            cudaEventRecord(e0, B->stream);
            rc = lbm_batch_step(&view, steps_per_trial);
            cudaEventRecord(e1, B->stream);
            if (!rc && cudaEventSynchronize(e1) != cudaSuccess) rc = bfail(LBM_ERR_CUDA, "autotune timing failed");
            float ms = 0.f;
            if (!rc) cudaEventElapsedTime(&ms, e0, e1);
            total_ms[q] += ms;
        }
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
        // restore the members whatever happened
        for (size_t k = 0; k < saved.size(); ++k) {
            lbm_lattice* L = view.members[k];
            const Saved& sv = saved[k];
            cudaMemcpyAsync(L->buf[sv.cur], sv.f, size_t(9) * L->plane * L->esize,
                            cudaMemcpyDeviceToDevice, B->stream);
            cudaFreeAsync(sv.f, B->stream);
            L->cur = sv.cur;
            L->time = sv.time;
            L->steps = sv.steps;
            L->mom_valid = false;
            if (!rc) rc = lbm_set_tile(L, sv.v, sv.rows);
        }
        view.members.clear();                              // the view owns nothing
        if (view.d_members) cudaFree(view.d_members);
        if (view.d_tasks) cudaFree(view.d_tasks);
        view.d_members = nullptr;
        view.d_tasks = nullptr;
        drop_graphs(&view);
        if (cudaStreamSynchronize(B->stream) != cudaSuccess && !rc) rc = bfail(LBM_ERR_CUDA, "autotune restore");
        if (rc) return rc;
    }
    const int best = total_ms[0] < total_ms[1] ? 0 : 1;
    B->V = kCandidates[best];
    if (int rc = ensure_table(B)) return rc;
    if (cache_path) {
        char line[640];
        auto mlups = [&](double ms) { return ms > 0.0 ? cells * steps_per_trial / (ms * 1e3) : 0.0; };
        std::snprintf(line, sizeof(line),
                      "{\"key\": \"%s\", \"V\": %d, \"mlups_v2\": %.1f, \"mlups_v4\": %.1f, \"members\": %d}",
                      key.c_str(), B->V, mlups(total_ms[0]), mlups(total_ms[1]), int(B->members.size()));
        kept.push_back(line);
        FILE* fh = std::fopen(cache_path, "w");
        if (!fh) return bfail(LBM_ERR_INVALID_ARGUMENT, std::string("cannot write ") + cache_path);
        std::fprintf(fh, "{\"lbm_batch_autotune\": [\n");
        for (size_t k = 0; k < kept.size(); ++k) {
            std::string t = kept[k];
            while (!t.empty() && t.front() == ' ') t.erase(t.begin());
            std::fprintf(fh, "  %s%s\n", t.c_str(), k + 1 < kept.size() ? "," : "");
        }
        std::fprintf(fh, "]}\n");
        std::fclose(fh);
    }
    return LBM_OK;
}

}  // extern "C"
