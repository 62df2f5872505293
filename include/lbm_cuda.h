/*
 * lbm_cuda.h — C ABI of the GB300 (sm_103a) D2Q9 lattice-Boltzmann solver.
 *
 * This is the drop-in boundary for taktoa/chemsim's `src/lbm.rs` lattice
 * storage and `State::step`.  Every entry point is plain C: opaque handles,
 * plain pointers and sizes, `int` status codes.  The Rust `lbm-cuda` crate
 * (lbm-cuda/src/lib.rs) binds these with `extern "C"` declarations.
 *
 * Conventions
 *  - Status: 0 = LBM_OK, negative = LBM_ERR_*.  The message of the last error
 *    on the calling thread is returned by lbm_last_error_string().  The Rust
 *    side turns a negative status into a panic, as lbm.rs does with
 *    assert!/assert_eq! (src/lbm.rs:51-52,188,191; src/matrix.rs:26,33-36).
 *  - Host field layout is row-major `y*w + x`, the layout of
 *    `Matrix::new` / `Matrix::get_underlying` (src/matrix.rs:24-30,120-126):
 *    row = y, column = x.
 *  - Populations are structure-of-arrays: plane i (i = 0..8, the direction
 *    order of `D2Q9::directions`, src/lbm.rs:202-282) occupies
 *    f[i*w*h .. (i+1)*w*h), each plane row-major `y*w + x`.
 *  - A handle owns its device memory and one CUDA stream.  A handle is not
 *    thread-safe; separate handles are independent.
 *  - Float precision of the device storage is chosen at creation; host
 *    buffers are always f32 (f64 for the *_f64 entry points).
 */
#ifndef LBM_CUDA_H
#define LBM_CUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define LBM_OK                    0
#define LBM_ERR_INVALID_ARGUMENT (-1)
#define LBM_ERR_OUT_OF_MEMORY    (-2)
#define LBM_ERR_CUDA             (-3)
#define LBM_ERR_UNSTABLE         (-4) /* health check found NaN/Inf or f_eq[0] < 0 */
#define LBM_ERR_TIMEOUT          (-5) /* a bounded device-side wait expired       */
#define LBM_ERR_NOT_SUPPORTED    (-6)
#define LBM_ERR_STATE            (-7) /* call order violated (e.g. no data yet)  */

/* ---- storage precision --------------------------------------------------- */
#define LBM_F32      0 /* f32 populations (the reference's Scalar = f32, src/lbm.rs:13) */
#define LBM_F64      1 /* f64 populations: the FP64 run of the same kernel             */
#define LBM_F16DEV   2 /* IEEE half storing scaled (f_i - w_i), collided in f32        */
#define LBM_BF16DEV  3 /* bfloat16 storing scaled (f_i - w_i), collided in f32         */

/* ---- boundary / mode flags (OR them together) --------------------------- */
/* Per-axis treatment of a pull source that lies outside the lattice.        */
#define LBM_X_ZEROPAD   0x00 /* zeros enter (af::convolve2 DEFAULT, src/lbm.rs:722-724) */
#define LBM_X_PERIODIC  0x01
#define LBM_X_WALL      0x02 /* half-way bounce-back wall beyond x = -1/2 and w - 1/2 */
#define LBM_Y_ZEROPAD   0x00
#define LBM_Y_PERIODIC  0x04
#define LBM_Y_WALL      0x08
/* Solid-node treatment.                                                       */
#define LBM_SOLID_FULLWAY 0x00 /* reference: after streaming, populations of a solid
                                  node are reversed in place and the node collides
                                  like any other (src/lbm.rs:741-751, :694-714)     */
#define LBM_SOLID_HALFWAY 0x10 /* half-way bounce-back: a link whose source node is
                                  solid returns the cell's own opposite population;
                                  solid nodes keep their populations unchanged     */
/* Frame: how a lattice velocity c = (cx, cy) maps to a grid displacement.     */
#define LBM_FRAME_REF   0x00 /* lbm.rs: convolve2 with the transposed stencil moves
                                direction i by (drow, dcol) = (-cx, +cy)           */
#define LBM_FRAME_XY    0x20 /* c moves by (dcol, drow) = (+cx, +cy): x = column    */
/* Arithmetic.                                                                   */
#define LBM_FAST        0x40 /* FMA-contracted, algebraically simplified collision
                                instead of the reference's operation order        */
/* 16-bit deviation storage rounds collided values stochastically by default
 * (random bits from the stored pair's own f32 bits, so runs reproduce): round-to-nearest
 * repeats the same error step after step on a slowly changing field, and
 * those errors add up.  This flag selects round-to-nearest (faster, less
 * accurate over long runs).  Ignored by f32 and f64 storage.               */
#define LBM_ROUND_NEAREST 0x80

/* The exact lbm.rs semantics: zero-padded streaming, full-way bounce-back on
 * solid nodes, the reference frame, the reference's f32 operation order.     */
#define LBM_REFERENCE_FLAGS 0x00

/* ---- collision operators ------------------------------------------------ */
#define LBM_COLLISION_BGK 0 /* src/lbm.rs:345-370 */
#define LBM_COLLISION_TRT 1 /* src/lbm.rs:374-451 */

typedef struct lbm_lattice lbm_lattice;

/* Global health of a lattice, reduced on the device in f64.
 * Replaces State::is_unstable (src/lbm.rs:815-818) and Matrix::sum
 * (src/matrix.rs:138-140) used as conservation checks.                        */
typedef struct lbm_health {
    double  mass;            /* sum of rho over all cells                        */
    double  momentum_x;      /* sum of rho*u (lattice c-frame components)        */
    double  momentum_y;
    double  min_population;  /* min over cells and directions of f_i             */
    double  min_eq0;         /* min over cells of f_eq[0]; < 0 is is_unstable()   */
    int64_t nonfinite_count; /* populations that are NaN or +-Inf                */
    int64_t steps;           /* steps taken since creation / last set            */
    int32_t unstable;        /* 1 when min_eq0 < 0 or nonfinite_count > 0        */
    int32_t reserved;
} lbm_health;

/* Returns the message of the last failed call on this thread ("" if none). */
const char* lbm_last_error_string(void);

/* Library version as MAJOR*10000 + MINOR*100 + PATCH. */
int lbm_version(void);

/* ---- single lattice ------------------------------------------------------ */

/* Create a w x h lattice (1 <= w, h <= 262140).  Replaces D2Q9::new +
 * State::initial (src/lbm.rs:187-200, :679-692).  Populations start at rest equilibrium
 * (rho = 1, u = 0); time = 0; Discretization {dx = 1, dt = 1}; BGK(tau). */
int lbm_create(int w, int h, float tau, int precision, int flags,
               lbm_lattice** out);
int lbm_destroy(lbm_lattice* lat);

/* Discretization {delta_x, delta_t} (src/lbm.rs:75-86). */
int lbm_set_discretization(lbm_lattice* lat, float delta_x, float delta_t);

/* Collision operator: LBM_COLLISION_BGK uses tau (BGK { tau }, src/lbm.rs:345);
 * LBM_COLLISION_TRT uses (tau_plus, tau_minus) (TRT, src/lbm.rs:374-377).   */
int lbm_set_collision(lbm_lattice* lat, int kind, float tau, float tau_minus);

/* Populations <- compute_equilibrium(rho, (ux, uy)) (src/lbm.rs:43-71).
 * rho/ux/uy are host arrays of w*h floats, row-major y*w+x.               */
int lbm_init_equilibrium(lbm_lattice* lat, const float* rho,
                         const float* ux, const float* uy);

/* Whole-state copies (9*w*h values, SoA, see layout above).  Replace
 * Lattice::populations / populations_mut (src/lbm.rs:113-114).            */
int lbm_set_populations(lbm_lattice* lat, const float* f);
int lbm_get_populations(lbm_lattice* lat, float* f);
int lbm_set_populations_f64(lbm_lattice* lat, const double* f);
int lbm_get_populations_f64(lbm_lattice* lat, double* f);

/* Solid mask (w*h bytes, nonzero = solid), replaces State::geometry
 * (src/lbm.rs:99, :673).  Callable between steps, as LBMSim::handle does
 * (src/main.rs:77-89).  NULL clears the geometry.                         */
int lbm_set_geometry(lbm_lattice* lat, const uint8_t* solid);

/* Constant body force (Guo forcing), in the lattice c-frame.  No reference
 * counterpart (TODO.md:6 lists gravity as not done).                      */
int lbm_set_force(lbm_lattice* lat, float fx, float fy);

/* Advance nsteps time steps: stream -> bounce-back -> collide, time += dt
 * (State::step, src/lbm.rs:694-714), one fused kernel per step, replayed
 * from a CUDA graph.  Asynchronous on the handle's stream.               */
int lbm_step(lbm_lattice* lat, int nsteps);

/* As lbm_step; the last step also writes rho/u into the handle's device
 * moment buffers, so a following lbm_read_moments costs only the copy.   */
int lbm_step_moments(lbm_lattice* lat, int nsteps);

/* rho, u of the current populations (Lattice::density / velocity,
 * src/lbm.rs:117-149): rho = sum f_i, u = (1/rho) * sum f_i c_i (minus F/2
 * when a force is set).  on_device != 0: the three pointers are device
 * pointers.  Synchronises the handle's stream.                           */
int lbm_read_moments(lbm_lattice* lat, float* rho, float* ux, float* uy,
                     int on_device);
/* The same fields copied to host memory without waiting, for render loops:
 * they are staged on the device in the lattice's stream order (a
 * device-to-device copy), then copied to the host on a second stream, so
 * following steps run while that copy is in flight.  The host buffers
 * (pinned, for the copy to overlap) must stay valid and unread until
 * lbm_readback_wait returns.  Two device staging areas are used in turn, so
 * a readback is staged while the previous one's host copy is in flight; the
 * host copies run one after another on the second stream.                 */
int lbm_read_moments_async(lbm_lattice* lat, float* rho, float* ux, float* uy);
/* nsteps time steps whose last one writes rho/u straight into rho, ux, uy:
 * w*h floats each, row-major y*w+x, in memory the GPU addresses (device or
 * managed memory, or pinned host memory from cudaHostAlloc /
 * cudaHostRegister, which the kernel writes over the host link; pageable
 * host memory is rejected).  Nothing is staged or copied afterwards, so the
 * readback of a render loop costs the host-link bandwidth of the writes
 * alone (src/main.rs:138-177 reads rho/u after every frame).  Asynchronous:
 * lbm_readback_wait returns once the fields are written, and the handle's
 * device moment buffers are left alone.  No reference counterpart.        */
int lbm_step_moments_to(lbm_lattice* lat, int nsteps, float* rho, float* ux, float* uy);
int lbm_readback_wait(lbm_lattice* lat);

/* Health check (see lbm_health).  Synchronises the handle's stream.      */
int lbm_check(lbm_lattice* lat, lbm_health* out);

/* State::time (src/lbm.rs:671) and the number of steps taken.            */
int lbm_get_time(lbm_lattice* lat, float* time, int64_t* steps);

/* Run the handle's work on a caller-provided CUDA stream (cudaStream_t
 * passed as void*); NULL restores the handle's own stream.               */
int lbm_set_stream(lbm_lattice* lat, void* stream);
int lbm_synchronize(lbm_lattice* lat);

/* Device pointer of population plane i of the current state, and the
 * plane pitch in elements (for zero-copy consumers such as a renderer).   */
int lbm_device_populations(lbm_lattice* lat, void** base, int64_t* plane_stride,
                           int* row_pitch);

/* Health check (as lbm_check) of populations the caller already holds on the
 * device, for callers that cannot call cudaMalloc: render or game loops that
 * must not pay cudaMalloc's implicit device synchronisation, hosts that have
 * reserved all device memory for their own pool, plugin hosts that forbid
 * library allocations.  No counterpart in the reference.
 *   populations: plane 0 of 9 SoA planes of the given precision, rows of
 *   row_pitch elements, planes plane_stride elements apart (the layout
 *   lbm_device_populations returns); stream: cudaStream_t or NULL.
 * Allocates nothing: its scratch is a static 768 KiB device array that every
 * GPU loading this library holds until exit.  At most 268435456 cells
 * (16384 x 16384); larger lattices return LBM_ERR_INVALID_ARGUMENT.  The
 * first call in each CUDA context (a device's primary context, the new one
 * that follows cudaDeviceReset, or a context the caller made current)
 * resolves the array's device address in that context.  Not callable while
 * `stream` (or the legacy stream) is being captured: it copies its result to
 * the host and synchronises `stream`.  Calls share the array, so calls that
 * overlap on the GPU race; every call overwrites all of the scratch it
 * reads, so nothing needs clearing between calls.  out->steps is 0.        */
int lbm_check_device_noalloc(const void* populations, int precision, int w, int h,
                             int row_pitch, int64_t plane_stride, float delta_x,
                             float delta_t, void* stream, lbm_health* out);

/* Tile of the fused step: cells per thread along x (f32: 2, 4 or 8, default
 * 4; f64: 2; 16-bit: 4 or 8, default 8) and warps (rows) per block (1..8,
 * default 4); 0 keeps the default.
 * No reference counterpart (tuning knob of the GB300 kernel).            */
int lbm_set_tile(lbm_lattice* lat, int cells_per_thread, int rows_per_block);

/* ---- batches of independent lattices ----------------------------------- */
/* No reference counterpart: many lattices of uneven sizes and relaxation
 * times advanced together, each time step one kernel launch over the warp
 * work items (row, warp tile) of all members.                             */

typedef struct lbm_batch lbm_batch;

/* One member of a batch: size, tau, boundary flags (axes and solid mode;
 * the frame and LBM_FAST are the batch's), body force and an optional host
 * solid mask (w*h bytes, row-major y*w+x, nonzero = solid).              */
typedef struct lbm_desc {
    int w, h;
    float tau;
    int flags;
    float fx, fy;
    const uint8_t* solid;
} lbm_desc;

/* Creates n f32 member lattices (at rest equilibrium) that step together.
 * flags: LBM_FRAME_XY and/or LBM_FAST for every member.  Members run on the
 * batch's CUDA stream; reach them with lbm_batch_lattice and use any
 * single-lattice entry point on them (initialise, geometry, moments, check)
 * except lbm_set_stream.  Destroying the batch destroys its members.     */
int lbm_batch_create(int n, const lbm_desc* descs, int flags, lbm_batch** out);
int lbm_batch_destroy(lbm_batch* batch);
int lbm_batch_size(lbm_batch* batch, int* n);
int lbm_batch_lattice(lbm_batch* batch, int index, lbm_lattice** out);

/* Advances every member nsteps steps: one kernel launch per step covers
 * every member (runs of 16 steps replay a captured CUDA graph); each
 * member's time and step count advance as with lbm_step.  Asynchronous on
 * the batch's stream.                                                      */
int lbm_batch_step(lbm_batch* batch, int nsteps);
int lbm_batch_synchronize(lbm_batch* batch);
int lbm_batch_set_stream(lbm_batch* batch, void* stream);

/* The batch's warp-tile width: 2 or 4 cells per thread (default 4), one
 * batch kernel each.  Batch steps run every member at this width; a member
 * set to another one with lbm_set_tile is set back at the next batch step.
 * Results do not depend on it.                                             */
int lbm_batch_set_tile(lbm_batch* batch, int cells_per_thread);
int lbm_batch_tile(lbm_batch* batch, int* cells_per_thread);

/* Picks the batch's tile width by timing both candidates on the members,
 * one width class (<= 96, <= 192, <= 384, <= 768, wider) at a time, whose
 * state (populations, time, step count) is saved before and restored after;
 * applies it and caches the choice in the JSON file cache_path (NULL: no
 * cache).  A cached entry for this GPU and mode is reused without timing.
 * steps_per_trial <= 0 selects 24.                                         */
int lbm_batch_autotune(lbm_batch* batch, const char* cache_path, int steps_per_trial);

/* ---- checkpoint / resume --------------------------------------------------
 * A 96-byte header (magic "LBMSTATE", version 1, w, h, precision, flags,
 * collision, has_solid, tau, tau_minus, dx, dt, fx, fy, time, steps), then
 * the nine population planes in the lattice's storage type (row-major
 * y * w + x; 16-bit storage keeps its raw deviation values, so save -> load
 * is exact), then the w * h solid mask when there is one.  lbm_load needs a
 * lattice of the same size, precision and boundary flags and restores its
 * state, geometry, force, collision, discretization, LBM_FAST, time and step
 * count.                                                                     */
int lbm_save(lbm_lattice* lat, const char* path);
int lbm_load(lbm_lattice* lat, const char* path);

/* ---- colour map (src/render.rs) ------------------------------------------
 * Renders the lattice's moments into an RGBA8 image of w x h pixels, pixel
 * (x, y) at byte (y * w + x) * 4, alpha 255, the way render_scalar_field /
 * render_vector_field (src/render.rs:23-207) colour a field: value =
 * logistic(z-score over all cells), hue 0 and saturation 1 for the scalar
 * modes, hue = (atan2(vy, vx) + pi) / 2pi and saturation 0.8 for the vector
 * modes (z-score of vx^2 + vy^2), HSV -> RGB, channel = clamp(round(256 c)).
 * With geometry_overlay, solid cells are (0, 0, 255) as in render_geometry
 * (src/render.rs:7-21).  Momentum density is rho * u of the moments.
 * rgba is a device pointer when on_device, else host memory.               */
#define LBM_RENDER_DENSITY 0
#define LBM_RENDER_SPEED 1
#define LBM_RENDER_VELOCITY 2
#define LBM_RENDER_MOMENTUM 3
int lbm_render(lbm_lattice* lat, int mode, int geometry_overlay, uint8_t* rgba, int on_device);
/* The same frame copied to host memory without waiting, like
 * lbm_read_moments_async (its staging waits for every readback in flight):
 * rgba (pinned, for overlap) holds the frame once lbm_readback_wait returns. */
int lbm_render_async(lbm_lattice* lat, int mode, int geometry_overlay, uint8_t* rgba);

/* ---- learned coarse-grid correction --------------------------------------
 * No reference counterpart.  A 4-layer 3x3 convolutional network (channels
 * 4 -> 32 -> 32 -> 32 -> 9, GELU (tanh form), bf16 weights, f32 accumulation on the
 * tensor cores) maps a coarse lattice's fields to a correction of its 9
 * populations.  Tensors passed as float* are device pointers in NCHW f32:
 * inputs (batch, 4, h, w) = ((rho - 1) * s_rho, ux * s_u, uy * s_u, solid);
 * outputs / targets (batch, 9, h, w).                                        */

typedef struct lbm_cnn lbm_cnn;

/* h x w images (w a multiple of 128), up to max_batch per call; weights
 * initialised from splitmix64(seed).                                        */
int lbm_cnn_create(int h, int w, int max_batch, uint64_t seed, lbm_cnn** out);
int lbm_cnn_destroy(lbm_cnn* net);
int lbm_cnn_param_count(lbm_cnn* net, int64_t* n);
/* All parameters as one f32 host array: per layer l = 0..3 the weights
 * W[tap = ky*3 + kx][cin][cout] followed by the biases[cout].              */
int lbm_cnn_get_params(lbm_cnn* net, float* params);
int lbm_cnn_set_params(lbm_cnn* net, const float* params);
int lbm_cnn_forward(lbm_cnn* net, const float* in, int batch, float* out);
/* Mean-squared-error loss against target and its gradient wrt every
 * parameter (grads: host array of param_count floats, or NULL).            */
int lbm_cnn_gradients(lbm_cnn* net, const float* in, const float* target, int batch,
                      float* loss, float* grads);
/* One Adam step (beta1 0.9, beta2 0.999) on the MSE loss.                  */
int lbm_cnn_train_step(lbm_cnn* net, const float* in, const float* target, int batch,
                       float lr, float* loss);
/* Diagnostic of the bounded device waits: one warp waits on an mbarrier that
 * nothing signals, giving up after `polls` polls (1 .. 4194304; each poll
 * sleeps about 32 ns) through the same routine the tensor-core kernels use,
 * and *timed_out reports that it gave up.  The context stays usable: this is
 * the path a lost arrival takes (those kernels then return LBM_ERR_TIMEOUT). */
int lbm_selftest_wait_timeout(uint32_t polls, int* timed_out);
/* Weights to / from a file: "LBMCNN01", int64 parameter count, the f32
 * parameters in lbm_cnn_get_params order.                                  */
int lbm_cnn_save(lbm_cnn* net, const char* path);
int lbm_cnn_load(lbm_cnn* net, const char* path);
/* Issue the net's work on `stream` (a cudaStream_t; NULL = the net's own
 * stream).  Calls read their input tensors in that stream's order, so a
 * caller that fills them on another stream orders the two itself.          */
int lbm_cnn_set_stream(lbm_cnn* net, void* stream);
int lbm_cnn_synchronize(lbm_cnn* net);

/* Fine -> coarse lattice (both f32; coarse sides = fine sides / factor):
 * coarse populations = f_eq of the block-averaged fine rho and momentum.   */
int lbm_restrict(lbm_lattice* fine, lbm_lattice* coarse, int factor);
/* The network input of a lattice as image `image` of a device tensor
 * (batch, 4, h, w) f32.                                                     */
int lbm_coarse_features(lbm_lattice* lat, float s_rho, float s_u, int image, float* in);
/* f_i += d_i - w_i * sum_j d_j with d_i = scale * corr[image][i] (each
 * clamped to +-max_abs when max_abs > 0) on the fluid cells of an f32
 * lattice: the correction never changes a cell's mass.                     */
int lbm_coarse_apply(lbm_lattice* lat, const float* corr, int image, float scale, float max_abs);
/* target[image][i] = (f_eq_i(rho_cur, u_ref) - f_eq_i(rho_cur, u_cur)) / scale
 * with u = j / rho of the stored states, zero on cur's solid cells, for two
 * f32 lattices of one size (ref holding equilibria, as lbm_restrict writes
 * them): the population change that moves cur's velocity onto ref's and
 * leaves its density and non-equilibrium part alone.                        */
int lbm_coarse_target(lbm_lattice* ref, lbm_lattice* cur, float scale, int image, float* target);
/* The learned coarse run: nsteps steps of an f32 lattice of the network's
 * size; after every k steps the network maps the lattice's features
 * (s_rho, s_u as in lbm_coarse_features) to a correction applied with
 * lbm_coarse_apply(scale, max_abs).  Every check_every corrections (0 =
 * never) a health check runs; if the lattice is unstable or its mass moved by
 * more than mass_tolerance (relative), the run stops and *fallback_step is
 * the lattice's step count at that point (the caller continues on the fine
 * grid), else *fallback_step = -1.  All work is on the lattice's stream.     */
int lbm_coarse_run(lbm_lattice* lat, lbm_cnn* net, int nsteps, int k, float s_rho, float s_u,
                   float scale, float max_abs, int check_every, float mass_tolerance,
                   int64_t* fallback_step);

#ifdef __cplusplus
}
#endif

#endif /* LBM_CUDA_H */
