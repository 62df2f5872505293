// lbm_batch.cu — many independent lattices advanced together.
//
// A batch owns n ordinary lattices (lbm_lattice handles, so every
// single-lattice entry point works on a member) and advances all of them by
// one persistent launch per time step: the grid is sized to fill the GPU
// once, and each warp walks the list of work items (member, row, warp tile)
// of all members, running the same interior / general step code as a single
// lattice, so a member's results do not depend on whether it was stepped
// alone or in a batch.  Runs of steps replay a captured CUDA graph.  The
// autotuner picks the tile width (cells per thread) per width class.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "lbm_handle.cuh"

using namespace lbmk;

struct lbm_batch_member_dev {
    StepArgs<float> a[2];   // from the member's buffer at build time (0) or the other (1)
    int V;                  // cells per thread
    int rows;               // warp rows per task
};

struct lbm_batch {
    std::vector<lbm_lattice*> members;
    std::vector<uint64_t> built_version;
    std::vector<int> built_cur;
    lbm_batch_member_dev* d_members = nullptr;
    uint2* d_tasks = nullptr;         // work items (member, row << 12 | tile), 4 lists
    int list_off[7] = {0, 0, 0, 0, 0, 0, 0};
    int ntasks = 0;
    size_t tasks_cap = 0;
    int par = 0;                      // steps since the table was built, mod 2
    bool built = false;
    int frame = 0, fast = 1;
    int grid[6] = {0, 0, 0, 0, 0, 0};  // per list: resident blocks of its kernel x SMs
    int grid_fused = 0;               // the same for the fused kernel
    cudaStream_t own = nullptr, stream = nullptr;
    cudaGraphExec_t graph[2] = {nullptr, nullptr};
    int dev = 0;
    bool owns = true;                 // destroys its members (false: a tuning view)
};

namespace {

constexpr int kTaskWarps = 8;
constexpr int kBatchGraphSteps = 16;

// Blocks of 8 warps per SM: 3 for the narrow-tile interior kernel, 2 (128
// registers a thread) for the others.  The member's arguments are read from memory,
// so collision constants live in registers.
#ifndef LBM_BATCH_MIN_BLOCKS
#define LBM_BATCH_MIN_BLOCKS 3
#endif
#ifndef LBM_BATCH_PREFETCH
#define LBM_BATCH_PREFETCH 1
#endif
// 1: every step is one launch of the fused kernel over all items; 0 (the
// default): one launch per non-empty list, each of its own kernel.  A/B on
// one GB300 (512 members, 154 M cells, autotuned): fused 0.566 of the copy
// bandwidth, lists 0.680.  The fused kernel takes the registers of its
// largest path (the general step, 128 a thread), so the lean items, which
// need 80, run at two thirds of their occupancy.
#ifndef LBM_BATCH_FUSED
#define LBM_BATCH_FUSED 0
#endif

// One warp = one work item; a warp walks its item list with a stride of the
// whole grid, fetching the next item before it works on the current one, and
// reads its member's step arguments straight from the (L1/L2-resident) member
// table, so warps never wait for one another.  Item word x = member index,
// word y = row << 12 | tile.  Each kernel carries one code path (the items
// are split by tile width and by the tile flag: PATH 1 = the full boundary /
// solid treatment, 2 = the interior step that wraps at periodic edges, 0 =
// the lean interior step), which keeps the instruction working set of an SM
// small.
template <int V, int FRAME, bool FAST, int PATH>
__global__ void __launch_bounds__(256, (PATH == 1 || V == 4) ? 2 : LBM_BATCH_MIN_BLOCKS)
lbm_batch_kernel(const lbm_batch_member_dev* __restrict__ members, const uint2* __restrict__ items,
                 int nitems, int parity) {
    const int lane = threadIdx.x;
    const int warps = gridDim.x * blockDim.y;
    int it = blockIdx.x * blockDim.y + threadIdx.y;
    uint2 item = it < nitems ? items[it] : make_uint2(0u, 0u);
    for (; it < nitems; it += warps) {
        const uint2 next = it + warps < nitems ? items[it + warps] : make_uint2(0u, 0u);
        if (LBM_BATCH_PREFETCH && lane < 9 && it + warps < nitems) {
            // L2 prefetch of the rows the next item pulls, one plane a lane
            // (the range is clipped to the row's pitch, so it stays inside
            // the member's buffer)
            const StepArgs<float>& an = members[next.x & 0xffffffu].a[parity];
            const int ys = int(next.y >> 12) - DROW(FRAME, lane);
            const int x0 = int(next.y & 4095u) * 32 * V;
            if (ys >= 0 && ys < an.h) {
                const int n = min(32 * V, an.pitch - x0);
                const float* p = static_cast<const float*>(an.src) + lane * an.plane +
                                 int64_t(ys) * an.pitch + x0;
                asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" :: "l"(p), "r"(n * 4) : "memory");
            }
        }
        const StepArgs<float>& a = members[item.x & 0xffffffu].a[parity];
        const int y = int(item.y >> 12), tile = int(item.y & 4095u);
        if constexpr (PATH == 1) step_general<float, V, FRAME, FAST>(a, y, tile, lane);
        else if constexpr (PATH == 2) step_interior_wrap<float, V, FRAME, FAST>(a, y, (tile * 32 + lane) * V, lane);
        else step_interior<float, V, FRAME, FAST>(a, y, (tile * 32 + lane) * V, lane);
        item = next;
    }
}

// All item kinds in one persistent kernel: item word x carries the member
// index in its low 24 bits and the list (tile width and path) in bits 24-26,
// and the warp dispatches on it, so a step is one launch.  Lists stay in
// order (general items first, so their longer latency overlaps the rest).
template <int FRAME, bool FAST>
__global__ void __launch_bounds__(256, 2)
lbm_batch_fused_kernel(const lbm_batch_member_dev* __restrict__ members,
                       const uint2* __restrict__ items, int nitems, int parity) {
    const int lane = threadIdx.x;
    const int warps = gridDim.x * blockDim.y;
    int it = blockIdx.x * blockDim.y + threadIdx.y;
    uint2 item = it < nitems ? items[it] : make_uint2(0u, 0u);
    for (; it < nitems; it += warps) {
        const uint2 next = it + warps < nitems ? items[it + warps] : make_uint2(0u, 0u);
        const int m = int(item.x & 0xffffffu), k = int(item.x >> 24);
        if (LBM_BATCH_PREFETCH && lane < 9 && it + warps < nitems) {
            const int nk = int(next.x >> 24), nv = nk < 3 ? 2 : 4;
            const StepArgs<float>& an = members[next.x & 0xffffffu].a[parity];
            const int ys = int(next.y >> 12) - DROW(FRAME, lane);
            const int x0 = int(next.y & 4095u) * 32 * nv;
            if (ys >= 0 && ys < an.h) {
                const int n = min(32 * nv, an.pitch - x0);
                const float* p = static_cast<const float*>(an.src) + lane * an.plane +
                                 int64_t(ys) * an.pitch + x0;
                asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" :: "l"(p), "r"(n * 4) : "memory");
            }
        }
        const StepArgs<float>& a = members[m].a[parity];
        const int y = int(item.y >> 12), tile = int(item.y & 4095u);
        switch (k) {     // warp-uniform
            case 0: step_general<float, 2, FRAME, FAST>(a, y, tile, lane); break;
            case 1: step_interior_wrap<float, 2, FRAME, FAST>(a, y, (tile * 32 + lane) * 2, lane); break;
            case 2: step_interior<float, 2, FRAME, FAST>(a, y, (tile * 32 + lane) * 2, lane); break;
            case 3: step_general<float, 4, FRAME, FAST>(a, y, tile, lane); break;
            case 4: step_interior_wrap<float, 4, FRAME, FAST>(a, y, (tile * 32 + lane) * 4, lane); break;
            default: step_interior<float, 4, FRAME, FAST>(a, y, (tile * 32 + lane) * 4, lane); break;
        }
        item = next;
    }
}

using BatchKernel = void (*)(const lbm_batch_member_dev*, const uint2*, int, int);

BatchKernel pick_fused(int frame, int fast) {
    if (frame) return fast ? lbm_batch_fused_kernel<1, true> : lbm_batch_fused_kernel<1, false>;
    return fast ? lbm_batch_fused_kernel<0, true> : lbm_batch_fused_kernel<0, false>;
}

template <int V, int PATH>
BatchKernel pick_kernel_v(int frame, int fast) {
    if (frame) return fast ? lbm_batch_kernel<V, 1, true, PATH> : lbm_batch_kernel<V, 1, false, PATH>;
    return fast ? lbm_batch_kernel<V, 0, true, PATH> : lbm_batch_kernel<V, 0, false, PATH>;
}

// List k = 3 * (V == 4) + j with j = 0 general, 1 periodic edge, 2 lean.
constexpr int kLists = 6;
BatchKernel pick_kernel(int list, int frame, int fast) {
    switch (list) {
        case 0: return pick_kernel_v<2, 1>(frame, fast);
        case 1: return pick_kernel_v<2, 2>(frame, fast);
        case 2: return pick_kernel_v<2, 0>(frame, fast);
        case 3: return pick_kernel_v<4, 1>(frame, fast);
        case 4: return pick_kernel_v<4, 2>(frame, fast);
        default: return pick_kernel_v<4, 0>(frame, fast);
    }
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

// (Re)builds the device member table and the task list when a member changed.
int ensure_table(lbm_batch* B) {
    const int n = int(B->members.size());
    bool changed = !B->built;
    for (int i = 0; i < n && !changed; ++i) {
        const lbm_lattice* L = B->members[i];
        if (L->version != B->built_version[i] || L->cur != (B->built_cur[i] ^ B->par)) changed = true;
    }
    if (!changed) return LBM_OK;
    std::vector<lbm_batch_member_dev> host(n);
    std::vector<uint2> lists[kLists];
    std::vector<uint8_t> flags;
    for (int i = 0; i < n; ++i) {
        lbm_lattice* L = B->members[i];
        host[i].a[0] = lattice_args<float>(L, L->cur, false);
        host[i].a[1] = lattice_args<float>(L, L->cur ^ 1, false);
        host[i].V = L->vcells;
        host[i].rows = L->rows;
        B->built_version[i] = L->version;
        B->built_cur[i] = L->cur;
        flags.resize(size_t(L->h) * L->ntiles);
        BATCH_CUDA(cudaMemcpyAsync(flags.data(), L->tflags, flags.size(), cudaMemcpyDeviceToHost,
                                   B->stream));
        BATCH_CUDA(cudaStreamSynchronize(B->stream));
        const int vbase = L->vcells == 2 ? 0 : 3;
        for (int r = 0; r < L->h; ++r)
            for (int t = 0; t < L->ntiles; ++t) {
                const uint8_t fl = flags[size_t(r) * L->ntiles + t];
                const int j = (fl & 1) ? 0 : (fl == 2 ? 1 : 2);     // 1, 3: general
                lists[vbase + j].push_back(make_uint2(uint32_t(i) | (uint32_t(vbase + j) << 24),
                                                      (uint32_t(r) << 12) | uint32_t(t)));
            }
    }
    std::vector<uint2> tasks;
    for (int k = 0; k < kLists; ++k) {
        B->list_off[k] = int(tasks.size());
        tasks.insert(tasks.end(), lists[k].begin(), lists[k].end());
    }
    B->list_off[kLists] = int(tasks.size());
    if (!B->d_members) BATCH_CUDA(cudaMalloc(&B->d_members, sizeof(lbm_batch_member_dev) * n));
    BATCH_CUDA(cudaMemcpyAsync(B->d_members, host.data(), sizeof(lbm_batch_member_dev) * n,
                               cudaMemcpyHostToDevice, B->stream));
    if (tasks.size() > B->tasks_cap) {
        if (B->d_tasks) cudaFree(B->d_tasks);
        B->d_tasks = nullptr;
        B->tasks_cap = 0;
        BATCH_CUDA(cudaMalloc(&B->d_tasks, sizeof(uint2) * tasks.size()));
        B->tasks_cap = tasks.size();
    }
    BATCH_CUDA(cudaMemcpyAsync(B->d_tasks, tasks.data(), sizeof(uint2) * tasks.size(),
                               cudaMemcpyHostToDevice, B->stream));
    BATCH_CUDA(cudaStreamSynchronize(B->stream));
    B->ntasks = int(tasks.size());
    B->par = 0;
    B->built = true;
    drop_graphs(B);
    return LBM_OK;
}

// One step: for each tile width, the general items, then the periodic-edge
// and the lean interior items, one launch per non-empty list.
cudaError_t launch(lbm_batch* B, int parity) {
    if (LBM_BATCH_FUSED) {
        if (B->ntasks == 0) return cudaSuccess;
        const int grid = std::min(B->grid_fused, (B->ntasks + kTaskWarps - 1) / kTaskWarps);
        pick_fused(B->frame, B->fast)<<<grid, dim3(32, kTaskWarps), 0, B->stream>>>(
            B->d_members, B->d_tasks, B->ntasks, parity);
        return cudaGetLastError();
    }
    for (int k = 0; k < kLists; ++k) {
        const int n = B->list_off[k + 1] - B->list_off[k];
        if (n == 0) continue;
        const int grid = std::min(B->grid[k], (n + kTaskWarps - 1) / kTaskWarps);
        pick_kernel(k, B->frame, B->fast)<<<grid, dim3(32, kTaskWarps), 0, B->stream>>>(
            B->d_members, B->d_tasks + B->list_off[k], n, parity);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
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

// Candidate tiles (cells per thread; the batch kernel's warp tile is 32 x
// that wide).  Rows per block only shapes a member's own launches.
const int kCandidates[][1] = {{2}, {4}};

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
    // Each list's persistent grid is exactly one wave of its own kernel: the
    // kernels differ in registers (2 or 3 resident blocks per SM), and a
    // second partial wave would leave SMs idle at the end of the launch.
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, B->dev);
    for (int k = 0; k < kLists; ++k) {
        int per_sm = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, pick_kernel(k, B->frame, B->fast),
                                                      32 * kTaskWarps, 0);
        B->grid[k] = std::max(1, sms) * std::max(1, per_sm);
    }
    {
        int per_sm = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, pick_fused(B->frame, B->fast),
                                                      32 * kTaskWarps, 0);
        B->grid_fused = std::max(1, sms) * std::max(1, per_sm);
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

int lbm_batch_autotune(lbm_batch* B, const char* cache_path, int steps_per_trial) {
    if (!B) return bfail(LBM_ERR_INVALID_ARGUMENT, "null batch");
    if (steps_per_trial <= 0) steps_per_trial = 24;
    cudaDeviceProp prop;
    BATCH_CUDA(cudaGetDeviceProperties(&prop, B->dev));
    char keybuf[320];
    std::snprintf(keybuf, sizeof(keybuf), "%s|f32|%s|%s", prop.name, B->frame ? "xy" : "ref",
                  B->fast ? "fast" : "strict");
    const std::string key(keybuf);
    const int ncand = int(sizeof(kCandidates) / sizeof(kCandidates[0]));
    int choice[5][2];
    bool have[5] = {false, false, false, false, false};
    // cached choices: one JSON object per line, {"key": "...", "class": c, "V": v, "rows": r, ...}
    std::vector<std::string> kept;
    if (cache_path) {
        if (FILE* fh = std::fopen(cache_path, "r")) {
            char line[1024];
            while (std::fgets(line, sizeof(line), fh)) {
                const char* k = std::strstr(line, "\"key\": \"");
                if (!k) continue;
                k += 8;
                const char* ke = std::strchr(k, '"');
                if (!ke) continue;
                std::string lk(k, ke - k);
                int c = -1, v = 0, r = 0;
                const char* pc = std::strstr(line, "\"class\": ");
                const char* pv = std::strstr(line, "\"V\": ");
                const char* pr = std::strstr(line, "\"rows\": ");
                if (pc) c = std::atoi(pc + 9);
                if (pv) v = std::atoi(pv + 5);
                if (pr) r = std::atoi(pr + 8);
                std::string body(line);
                while (!body.empty() && (body.back() == '\n' || body.back() == ',' || body.back() == ' '))
                    body.pop_back();
                if (lk == key && c >= 0 && c < 5 && (v == 2 || v == 4) && (r == 1 || r == 2 || r == 4 || r == 8)) {
                    choice[c][0] = v;
                    choice[c][1] = r;
                    have[c] = true;
                } else if (body.find("\"key\"") != std::string::npos) {
                    kept.push_back(body);
                }
            }
            std::fclose(fh);
        }
    }
    bool needed[5] = {false, false, false, false, false};
    for (lbm_lattice* L : B->members) needed[width_class(L->w)] = true;
    std::vector<std::string> timed;
    for (int c = 0; c < 5; ++c) {
        if (!needed[c] || have[c]) continue;
        // Time the class's own members through a non-owning view of them,
        // with their state saved first and restored afterwards.
        lbm_batch view;
        view.owns = false;
        view.frame = B->frame;
        view.fast = B->fast;
        std::copy(B->grid, B->grid + kLists, view.grid);
        view.grid_fused = B->grid_fused;
        view.stream = B->stream;
        view.dev = B->dev;
        struct Saved { void* f; int cur; float time; int64_t steps; int v, rows; };
        std::vector<Saved> saved;
        double cells = 0.0;
        int rc = LBM_OK;
        for (lbm_lattice* L : B->members) {
            if (width_class(L->w) != c) continue;
            Saved sv{nullptr, L->cur, L->time, L->steps, L->vcells, L->rows};
            const size_t bytes = size_t(9) * L->plane * L->esize;
            cudaError_t e = cudaMallocAsync(&sv.f, bytes, B->stream);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(sv.f, L->buf[L->cur], bytes, cudaMemcpyDeviceToDevice, B->stream);
            if (e != cudaSuccess) { rc = bfail(LBM_ERR_CUDA, cudaGetErrorString(e)); (void)cudaGetLastError(); break; }
            saved.push_back(sv);
            view.members.push_back(L);
            view.built_version.push_back(~uint64_t(0));
            view.built_cur.push_back(0);
            cells += double(L->w) * L->h;
        }
        float best = 1e30f;
        int bv = 4;
        cudaEvent_t e0 = nullptr, e1 = nullptr;
        if (!rc) { cudaEventCreate(&e0); cudaEventCreate(&e1); }
        for (int q = 0; q < ncand && !rc; ++q) {
            for (lbm_lattice* L : view.members)
                if ((rc = lbm_set_tile(L, kCandidates[q][0], L->rows))) break;
            if (!rc) rc = lbm_batch_step(&view, 4);
            if (rc) break;
            cudaEventRecord(e0, B->stream);
            rc = lbm_batch_step(&view, steps_per_trial);
            cudaEventRecord(e1, B->stream);
            if (!rc && cudaEventSynchronize(e1) != cudaSuccess) rc = bfail(LBM_ERR_CUDA, "autotune timing failed");
            float ms = 0.f;
            if (!rc) cudaEventElapsedTime(&ms, e0, e1);
            if (!rc && ms < best) { best = ms; bv = kCandidates[q][0]; }
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
        choice[c][0] = bv;
        choice[c][1] = 4;
        have[c] = true;
        char line[640];
        std::snprintf(line, sizeof(line),
                      "  {\"key\": \"%s\", \"class\": %d, \"V\": %d, \"rows\": %d, "
                      "\"mlups\": %.1f, \"members\": %d}",
                      key.c_str(), c, bv, 4, cells * steps_per_trial / (double(best) * 1e3),
                      int(saved.size()));
        timed.push_back(line);
    }
    for (lbm_lattice* L : B->members) {
        const int c = width_class(L->w);
        if (int rc = lbm_set_tile(L, choice[c][0], choice[c][1])) return rc;
    }
    if (cache_path && !timed.empty()) {
        // rewrite: other keys kept, this key's classes (cached + new) written
        for (int c = 0; c < 5; ++c) {
            if (!have[c]) continue;
            bool is_new = false;
            for (const auto& t : timed)
                if (t.find("\"class\": " + std::to_string(c) + ",") != std::string::npos) is_new = true;
            if (is_new) continue;
            char line[640];
            std::snprintf(line, sizeof(line), "  {\"key\": \"%s\", \"class\": %d, \"V\": %d, \"rows\": %d}",
                          key.c_str(), c, choice[c][0], choice[c][1]);
            kept.push_back(line);
        }
        for (auto& t : timed) kept.push_back(t);
        FILE* fh = std::fopen(cache_path, "w");
        if (!fh) return bfail(LBM_ERR_INVALID_ARGUMENT, std::string("cannot write ") + cache_path);
        std::fprintf(fh, "{\"lbm_batch_autotune\": [\n");
        for (size_t k = 0; k < kept.size(); ++k) {
            std::string s = kept[k];
            while (!s.empty() && s.front() == ' ') s.erase(s.begin());
            std::fprintf(fh, "  %s%s\n", s.c_str(), k + 1 < kept.size() ? "," : "");
        }
        std::fprintf(fh, "]}\n");
        std::fclose(fh);
    }
    return LBM_OK;
}

}  // extern "C"
