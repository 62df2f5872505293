// lbm_handle.cuh — the lattice handle shared by the single-lattice and the
// batched entry points (host-side, internal to liblbm_cuda.so).
#pragma once

#include <string>

#include "lbm_aux.cuh"

struct lbm_lattice {
    int w = 0, h = 0, precision = 0, flags = 0;
    int pitch = 0, mpitch = 0;
    int64_t plane = 0;
    size_t esize = 0;
    void* buf[2] = {nullptr, nullptr};
    int cur = 0;
    uint8_t* solid = nullptr;
    bool has_solid = false;
    float* mom[3] = {nullptr, nullptr, nullptr};
    bool mom_valid = false;
    void* staging = nullptr;
    size_t staging_bytes = 0;
    lbmk::HealthPartial* health = nullptr;  // kHealthBlocks partials + 1 result
    void* render = nullptr;               // colour-map scratch (stats, host-bound image)
    size_t render_bytes = 0;
    float* rb[2] = {nullptr, nullptr};    // staged moments of asynchronous readbacks, used in turn
    cudaEvent_t rb_done[2] = {nullptr, nullptr};  // the host copy out of rb[i] has finished
    bool rb_used[2] = {false, false};     // rb_done[i] has been recorded
    int rb_next = 0;                      // staging area of the next readback
    cudaStream_t rb_stream = nullptr;     // their device-to-host copies
    cudaEvent_t rb_staged = nullptr, rb_landed = nullptr;   // rb_landed: the latest readback landed
    bool rb_pending = false;
    uint8_t* tflags = nullptr;            // h x ceil(w / 32) bytes
    int ntiles = 0;
    uint32_t* gtiles = nullptr;           // list of flagged tiles
    int ngtiles = 0;
    size_t gtiles_cap = 0;
    uint4* links = nullptr;               // per (tile, lane) link masks (16-bit storage, 8 cells)
    size_t links_cap = 0;                 // in uint4 entries
    bool use_links = false;               // tiles flagged 3 run in the grid with the link masks
    int collision = LBM_COLLISION_BGK;
    float tau = 1.f, tau_minus = 1.f, dx = 1.f, dt = 1.f, fx = 0.f, fy = 0.f;
    float time = 0.f;
    int64_t steps = 0;
    cudaStream_t own = nullptr, stream = nullptr;
    cudaGraphExec_t graph[2] = {nullptr, nullptr};
    bool dirty = true;                    // captured graphs are stale
    uint64_t version = 0;                 // bumped on every change of the step arguments
    int vcells = 0, rows = 4;
    int dev = 0;
};

namespace lbmk {

// Step arguments of lattice L from buffer `from` (moments written when asked).
template <class S>
StepArgs<typename Store<S>::CT> lattice_args(const lbm_lattice* L, int from, bool moments);

// Bookkeeping after nsteps steps run by someone else (the batch kernel):
// buffer parity, State::time, the step count and the moment cache.
void lattice_advance(lbm_lattice* L, int nsteps);

// Brings L's moment buffers (rho, ux, uy) up to date with its state.
int lattice_refresh_moments(lbm_lattice* L);

// Creates the stream and events of asynchronous readbacks (once).
int lattice_readback_stream(lbm_lattice* L);

// Records msg for lbm_last_error_string and returns code.
int lattice_fail(int code, const std::string& msg);

}  // namespace lbmk
