/*
 * cardiax_gb300 -- C ABI of the GB300 Fenton-Karma stepper.
 *
 * Plain pointers and sizes only.  Every device pointer is a CUDA device address; `stream` is a
 * cudaStream_t (NULL = the legacy default stream).  No entry point allocates device memory.
 * Callers pass every buffer, including the ping-pong scratch state -- except for
 * fk_forward_euler_noalloc, whose scratch state is a fixed-size device array owned by the
 * library (see its declaration for the limit and the sharing rules).
 *
 * Layout
 *   A grid is H rows x W columns of float32 with a row pitch of `pitch` elements
 *   (pitch >= W, pitch % 4 == 0, base addresses 16-byte aligned).  A state is three such planes
 *   back to back -- v, w, u, the field order of the reference's State (cardiax/solve.py:12-15) --
 *   so plane p starts at state + p * H * pitch.  The diffusivity map and dense stimulus fields
 *   are single planes with the same pitch.
 *
 * Time
 *   Steps are integers; the stimulus protocol is evaluated on the float32 step index exactly as
 *   the reference's loop does (cardiax/solve.py:92-100, 262-267).
 *
 * Errors
 *   Every entry point returns FK_OK (0) or a positive fk_status code; fk_status_string() names
 *   it.  Launch errors are reported synchronously; device-side barrier timeouts set a sticky
 *   word read by fk_device_status().
 */
#ifndef CARDIAX_GB300_H
#define CARDIAX_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    FK_OK = 0,
    FK_ERR_NULL = 1,       /* a required pointer is NULL                          */
    FK_ERR_SHAPE = 2,      /* H or W < 3, pitch < W, or sizes out of range         */
    FK_ERR_ALIGN = 3,      /* pitch % 4 != 0 or a pointer is not 16-byte aligned   */
    FK_ERR_STIMULI = 4,    /* too many stimuli or an invalid protocol              */
    FK_ERR_ARGUMENT = 5,   /* any other invalid argument (dx <= 0, t1 < t0, ...)   */
    FK_ERR_CUDA = 6,       /* a CUDA call failed                                   */
    FK_ERR_TENSORMAP = 7,  /* the TMA descriptor could not be encoded              */
    FK_ERR_DEVICE = 8,     /* a kernel reported a barrier timeout                  */
    FK_ERR_CAPACITY = 9    /* grid larger than fk_forward_euler_noalloc's scratch  */
} fk_status;

/* The 14 Fenton-Karma parameters in the reference's field order (cardiax/params.py:4-18). */
typedef struct {
    float tau_v_plus, tau_v1_minus, tau_v2_minus, tau_w_plus, tau_w_minus;
    float tau_d, tau_0, tau_r, tau_si, k, V_csi, V_c, V_v, Cm;
} fk_params;

/* One stimulus (cardiax/stimulus.py:13-21).  Protocol values are in steps.  The field is
 * either dense (`field` != NULL, one plane with the grid's pitch) or, when `field` is NULL, the
 * rectangle [r0, r1) x [c0, c1) of value `amplitude` and zero elsewhere.  Where active stimuli
 * overlap, the later one in the list wins; a zero field value leaves the ionic current. */
typedef struct {
    double start, duration, period;
    const float *field;
    int32_t r0, r1, c0, c1;
    float amplitude;
} fk_stimulus;

/* A call takes up to FK_MAX_STIMULI stimuli.  At most FK_MAX_ACTIVE_STIMULI of them may be
 * active at any one step of a call that launches one kernel per step (fk_step, fk_euler_step,
 * fk_forward_euler[_tracked], fk_forward, fk_heun_step, fk_forward_heun, and the one-step
 * remainder of fk_forward_euler_tb): the library passes each launch the stimuli active at its
 * step, in list order.  Calls that advance several steps per launch (fk_forward_euler_tb,
 * fk_forward_euler_flow, fk_forward_flow, the batch and the adjoint) need the stimuli that can
 * be active anywhere in a launch's steps to number at most FK_MAX_ACTIVE_STIMULI (for the batch
 * and the adjoint: a tissue's whole list).  More: FK_ERR_STIMULI. */
#define FK_MAX_STIMULI 64
#define FK_MAX_ACTIVE_STIMULI 8

typedef struct {
    int64_t H, W, pitch;
} fk_grid;

/* Name of a status code. */
const char *fk_status_string(int status);

/* Reads (and with reset != 0 clears) the device error word of the current device. */
int fk_device_status(int reset, int *value);

/* Failure-path self-test: launches one warp that waits on a barrier nothing completes, with the
 * bounded wait the step kernels use cut to `limit_ns` (1 us .. 2 s); when it runs out the kernel
 * sets the device error word (read it with fk_device_status) and returns, leaving the context
 * usable.  No counterpart in the reference. */
int fk_selftest_wait_timeout(int64_t limit_ns, void *stream);

/* Which kernel takes the Euler steps of every single-tissue entry point (process-wide):
 * 0 = the tiled kernel (32 x 64-cell tiles, two passes) -- the default; 1 = the strip kernel
 * (128-column strips walked row by row with register windows) wherever it applies (W % 128 != 1),
 * else the tiled kernel.  Both produce the same bits; the switch exists to compare them.
 * No counterpart in the reference. */
int fk_select_step_kernel(int which);

/* init (cardiax/solve.py:18-23): v = w = 1, u = 0 on the three planes of `state`. */
int fk_init(fk_grid g, float *state, void *stream);

/* step (cardiax/solve.py:26-65): the time derivative (dv, dw, du) of `state` at step `t`,
 * written to `dstate` (a separate state buffer). */
int fk_step(fk_grid g, const float *state, const float *D, const fk_params *p,
            const fk_stimulus *stimuli, int n_stimuli, int64_t t, double dx, float *dstate,
            void *stream);

/* step_euler (cardiax/solve.py:68-70): one explicit Euler step from `state` at step `t` into
 * `state_out` (a separate buffer). */
int fk_euler_step(fk_grid g, const float *state, const float *D, const fk_params *p,
                  const fk_stimulus *stimuli, int n_stimuli, int64_t t, double dt, double dx,
                  float *state_out, void *stream);

/* _forward_euler (cardiax/solve.py:92-100): steps t0 .. t1-1 applied to `state` in place;
 * `scratch` is a second state buffer of the same size. */
int fk_forward_euler(fk_grid g, float *state, float *scratch, const float *D, const fk_params *p,
                     const fk_stimulus *stimuli, int n_stimuli, int64_t t0, int64_t t1,
                     double dt, double dx, void *stream);

/* fk_forward_euler without the scratch argument, for callers that cannot allocate device memory
 * (an XLA custom call, for instance, gets all of its buffers from XLA and must not allocate).
 * No counterpart in the reference.  The scratch state is a file-scope device array of this
 * library holding FK_NOALLOC_MAX_CELLS cells (H * pitch <= 512 * 512, 3 MiB per GPU for the
 * life of the process); larger grids return FK_ERR_CAPACITY.  The first call on a device, and
 * the first one after that device's context changed (a cudaDeviceReset, for instance), looks up
 * the array's address: make it before any stream capture.  Calls that overlap on the GPU share
 * the array and race.  Nothing needs clearing between calls: the in-grid cells of the result
 * never depend on earlier calls, and the state's row padding (columns W .. pitch-1) comes back
 * unchanged. */
#define FK_NOALLOC_MAX_CELLS (512 * 512)
int fk_forward_euler_noalloc(fk_grid g, float *state, const float *D, const fk_params *p,
                             const fk_stimulus *stimuli, int n_stimuli, int64_t t0, int64_t t1,
                             double dt, double dx, void *stream);

/* step_heun (cardiax/solve.py:73-85): x1 = x + dt f(x, t); out = x + (f(x, t) + f(x1, t)) dt/2,
 * both stages at step index t as in the reference.  `work` holds 3 state buffers. */
int fk_heun_step(fk_grid g, const float *state, const float *D, const fk_params *p,
                 const fk_stimulus *stimuli, int n_stimuli, int64_t t, double dt, double dx,
                 float *state_out, float *work, void *stream);

/* _forward_heun (cardiax/solve.py:103-111): Heun steps t0 .. t1-1 applied to `state` in place;
 * `work` holds 4 state buffers. */
int fk_forward_heun(fk_grid g, float *state, float *work, const float *D, const fk_params *p,
                    const fk_stimulus *stimuli, int n_stimuli, int64_t t0, int64_t t1, double dt,
                    double dx, void *stream);

/* forward (cardiax/solve.py:168-222): for i in 0 .. n_checkpoints-2, advances from
 * checkpoints[i] to checkpoints[i+1] and writes that state to out + i * 3 * H * pitch.
 * `state0` is only read; `scratch` is one state buffer.  Checkpoints must be non-decreasing. */
int fk_forward(fk_grid g, const float *state0, float *scratch, const float *D,
               const fk_params *p, const fk_stimulus *stimuli, int n_stimuli,
               const int64_t *checkpoints, int n_checkpoints, double dt, double dx, float *out,
               void *stream);

/* Activation-time maps (int32 planes with the grid's pitch).  An activation is an upstroke of u
 * through `threshold` during step t -> t+1; it is recorded as time t+1: `last` = t+1, `first` =
 * t+1 if it was negative, `count` += 1.  Initialise first/last to -1 and count to 0.  The
 * reference has no activation metric (its cardiax/metrics.py stubs are empty); these maps are
 * what long chaotic runs are compared on. */
typedef struct {
    int32_t *first, *last, *count;
    float threshold;
} fk_activation;

/* fk_forward_euler with activation tracking (`act` may be NULL: plain stepping). */
int fk_forward_euler_tracked(fk_grid g, float *state, float *scratch, const float *D,
                             const fk_params *p, const fk_stimulus *stimuli, int n_stimuli,
                             int64_t t0, int64_t t1, double dt, double dx,
                             const fk_activation *act, void *stream);

/* Temporal blocking (no reference counterpart; same results bit for bit): fk_forward_euler with
 * `depth` steps (1, 2, 4 or 8) per launch.  Each tile is loaded once with a 4*depth-cell halo,
 * advanced `depth` times in shared memory (recomputing the halo ring) and stored once; the last
 * (t1 - t0) mod depth steps, and grids whose last tile row or column is one cell wide (H % 32 or
 * W % 64 == 1; H % 16 or W % 16 == 1 at depth 8), run one step per launch. */
int fk_forward_euler_tb(fk_grid g, float *state, float *scratch, const float *D,
                        const fk_params *p, const fk_stimulus *stimuli, int n_stimuli, int64_t t0,
                        int64_t t1, double dt, double dx, int depth, void *stream);

/* Dataflow stepping: fk_forward_euler_tracked and fk_forward in one cooperative launch per call
 * instead of one launch per step (no reference counterpart; same results bit for bit).  Tile T of
 * step t starts as soon as T and its eight neighbours have finished step t-1, tracked in
 * `flags`: an int32 device array of at least fk_flow_flag_words(g) words owned by the call
 * (zeroed by the call on `stream`; calls that overlap on the GPU need separate arrays). */
int64_t fk_flow_flag_words(fk_grid g);

/* Steps t0 .. t1-1 from `src` into `dst` (src == dst: in place); `scratch` is a third state
 * buffer (distinct from src and dst) and `act` may be NULL. */
int fk_forward_euler_flow(fk_grid g, const float *src, float *dst, float *scratch,
                          const float *D, const fk_params *p, const fk_stimulus *stimuli,
                          int n_stimuli, int64_t t0, int64_t t1, double dt, double dx,
                          const fk_activation *act, int32_t *flags, int64_t n_flags,
                          void *stream);

/* fk_forward through the dataflow kernel (one launch per checkpoint interval). */
int fk_forward_flow(fk_grid g, const float *state0, float *scratch, const float *D,
                    const fk_params *p, const fk_stimulus *stimuli, int n_stimuli,
                    const int64_t *checkpoints, int n_checkpoints, double dt, double dx,
                    float *out, int32_t *flags, int64_t n_flags, void *stream);

/* ---- checkpoint emission ----------------------------------------------------------------------
 * io.imresize (cardiax/io.py:118-124), which the data-generation caller applies to every
 * checkpoint (deepx/generate.py:187-199): `planes` float32 planes of H x W (row pitch in_pitch,
 * planes H * in_pitch apart) resized to OH x OW (out_pitch, planes OH * out_pitch apart) with
 * the bilinear (triangle-kernel, half-pixel-centre) resampling of jax.image.resize, widened when
 * downsampling if `antialias` (jax.image.resize's default). */
int fk_resize_bilinear(const float *in, int64_t planes, int64_t H, int64_t W, int64_t in_pitch,
                       float *out, int64_t OH, int64_t OW, int64_t out_pitch, int antialias,
                       void *stream);

/* stimulus.triangular (cardiax/stimulus.py:109-140): the H x W plane `in` rotated by `angle_deg`
 * degrees about its centre into `out` (a separate plane) as scipy.ndimage.rotate(mode="nearest",
 * prefilter=False, reshape=False) does: order-3 B-spline of the samples, edge-replicated. */
int fk_rotate_field(const float *in, int64_t H, int64_t W, int64_t pitch, float *out,
                    int64_t out_pitch, double angle_deg, void *stream);

/* Scar maps (deepx/utils_scars.py:409-426 random_diffusivity_scar; the polygon outlines, random
 * draws and Gaussian weights are host work of a few hundred values).
 *
 * fk_scar_raster: the H x W plane `out` (pitch) set to 1 where a cell lies inside any of
 * `n_polys` <= 16 polygons and 0 elsewhere -- the union of skimage.draw.polygon fills of
 * utils_scars.py:79-97 clipped at 1 (utils_scars.py:356-360).  Polygon p has the vertices
 * (xs[k], ys[k]) for k in [offsets[p], offsets[p + 1]) (device arrays of doubles, x = column,
 * y = row; `offsets` is a HOST array of n_polys + 1 ints starting at 0, at least 3 vertices per
 * polygon, 4096 in all).  A cell (r, c) is inside when PNPOLY's crossing test holds at
 * (x = c, y = r), in double precision with separately rounded operations.  The number of cells
 * set is ADDED to *count (a device counter the caller zeroes). */
int fk_scar_raster(const double *xs, const double *ys, const int32_t *offsets, int64_t n_polys,
                   int64_t H, int64_t W, float *out, int64_t pitch, unsigned long long *count,
                   void *stream);

/* fk_conv2d_same: scipy.signal.convolve2d(in, kernel, "same") in float32 (the blur of
 * utils_scars.py:402-406): out[i][j] = sum over a, b < K of kernel[a * K + b] *
 * in[i + (K - 1) / 2 - a][j + (K - 1) / 2 - b], zero outside the plane; stored as 1 - out when
 * `one_minus` (utils_scars.py:426).  `kernel` is a device array of K * K floats; `in` and `out`
 * are distinct H x W planes (pitches in elements). */
int fk_conv2d_same(const float *in, int64_t H, int64_t W, int64_t in_pitch, const float *kernel,
                   int64_t K, float *out, int64_t out_pitch, int one_minus, void *stream);

/* ---- many tissues in one launch --------------------------------------------------------------
 * No reference counterpart: the reference steps one tissue per call (its data generation loops
 * over tissues in Python, deepx/generate.py:135-210).  Here every tissue of a batch advances in
 * one persistent kernel per step that drains a list of tiles of all tissues, and runs of
 * steps are replayed from a captured CUDA graph.  Tissues may differ in shape, parameters, D,
 * stimuli and dt/dx; they advance through the same step indices. */
typedef struct {
    fk_grid g;
    float *state;   /* (3, H, pitch), advanced in place                      */
    float *scratch; /* (3, H, pitch), ping-pong buffer                       */
    const float *D;
    fk_params params;
    const fk_stimulus *stimuli; /* copied at fk_batch_create             */
    int n_stimuli;
    double dt, dx;
    fk_activation act; /* act.last == NULL: no activation tracking       */
} fk_tissue;

typedef struct fk_batch fk_batch; /* opaque host-side plan */

/* Device workspace (bytes) that fk_batch_create needs for these tissues. */
size_t fk_batch_workspace_bytes(const fk_tissue *tissues, int n_tissues);

/* Validates the tissues, writes their descriptors, TMA maps and the tile list into `workspace`
 * (device memory of at least fk_batch_workspace_bytes, 128-byte aligned) on `stream`, and
 * returns a host-side plan.  The tissues' buffers must outlive the plan. */
int fk_batch_create(const fk_tissue *tissues, int n_tissues, void *workspace,
                    size_t workspace_bytes, void *stream, fk_batch **plan);

/* Advances every tissue through steps t0 .. t1-1.  graph_steps > 0 captures that many steps
 * (rounded up to even) into a CUDA graph once per plan and replays it; 0 launches each step. */
int fk_batch_forward_euler(fk_batch *plan, int64_t t0, int64_t t1, int graph_steps, void *stream);

/* Number of persistent CTAs per launch (default: two per SM); a tuning knob. */
int fk_batch_set_grid(fk_batch *plan, int ctas);

/* Tile geometry of the batched kernel: `rows` x 64-cell work items, rows = 32 (the default) or
 * 16.  Both give the same bits; the autotuner picks the faster for a batch.  No counterpart in
 * the reference. */
int fk_batch_set_tile_rows(fk_batch *plan, int rows);

/* Work order and arithmetic of the batched kernel: interleave = 1 (the default) deals the
 * work list round-robin to the CTAs (edge tiles first), 2, 4 or 8 deals it round-robin in chunks
 * of that many neighbouring items (a CTA's consecutive items then mostly share a tissue), 0 gives
 * each CTA a contiguous run of it (tissue by tissue, balanced by cost); other values:
 * FK_ERR_ARGUMENT.  packed != 0 uses packed two-cell FP32 instructions (default 0: scalar).
 * Same bits either way; tuning knobs.  No counterpart in the reference. */
int fk_batch_set_options(fk_batch *plan, int interleave, int packed);

/* Euler steps per launch of the batched path: 1 (the default), or 2 -- the temporally blocked
 * kernel on the 32 x 64 work items, each tile advanced two steps between one load and one store
 * (an odd last step runs alone).  Depth 2 needs every tissue's last tile row and column to hold
 * more than one cell (H % 32 != 1, W % 64 != 1) and no activation tracking; FK_ERR_ARGUMENT
 * otherwise.  Same bits either way.  No counterpart in the reference. */
int fk_batch_set_depth(fk_batch *plan, int depth);

int fk_batch_destroy(fk_batch *plan);

/* ---- reverse mode ---------------------------------------------------------------------------
 * Adjoint of fk_euler_step (cardiax/solve.py:68-70 through step, :26-65).  The reference never
 * differentiates its stepper (jax.grad of _forward_euler would fail on its while_loop); this is
 * the derivative that jax.grad of a scan of step_euler defines: Heaviside gates and the
 * stimulus replacement have zero derivative.
 *
 * Given state x_t (at step t) and the cotangent lam_next of x_{t+1}, writes the cotangent of
 * x_t to lam (a separate state buffer) and accumulates dL/dD into grad_D (one plane, +=) and
 * per-block partial sums of dL/dtheta into grad_theta_slots (+=; fk_adjoint_slots(g) slots of
 * 16 doubles; the first 13 are the parameters in cardiax Params order, Cm excluded).  Summing
 * the slots in index order gives a deterministic total.  grad_D / grad_theta_slots may be
 * NULL. */
int64_t fk_adjoint_slots(fk_grid g);
int fk_adjoint_step(fk_grid g, const float *state, const float *D, const fk_params *p,
                    const fk_stimulus *stimuli, int n_stimuli, int64_t t, double dt, double dx,
                    const float *lam_next, float *lam, float *grad_D, double *grad_theta_slots,
                    void *stream);

/* Segment helpers of a checkpointed reverse pass (one C call per segment instead of one per
 * step).  fk_recompute writes x_s (a copy of `state`) and x_{s+1} .. x_{s+n-1} into `buf`
 * (n consecutive states).  fk_adjoint_range walks k = n-1 .. 0: lam <- adjoint step at
 * x_{s+k} (buf[k]), then adds inj_grads[j] to lam for every j with inj_steps[j] == s+k.  On
 * entry lam is the cotangent of x_{s+n}; on return that of x_s.  lam_tmp is a second state
 * buffer.  Gradients accumulate as in fk_adjoint_step. */
int fk_recompute(fk_grid g, const float *state, int64_t s, int64_t n, const float *D,
                 const fk_params *p, const fk_stimulus *stimuli, int n_stimuli, double dt,
                 double dx, float *buf, void *stream);
int fk_adjoint_range(fk_grid g, const float *buf, int64_t s, int64_t n, const float *D,
                     const fk_params *p, const fk_stimulus *stimuli, int n_stimuli, double dt,
                     double dx, float *lam, float *lam_tmp, const int64_t *inj_steps,
                     const float *const *inj_grads, int n_inj, float *grad_D,
                     double *grad_theta_slots, void *stream);

/* Batched reverse pass: E experiments on one grid that share D and the parameters (each with
 * its own stimuli and state), as in an inverse problem fitted to several recordings.  No
 * reference counterpart.  Per experiment the results equal fk_recompute / fk_adjoint_range bit
 * for bit; every step is one launch for all experiments.
 *
 * fk_batch_recompute: `plan` holds the E experiments as its tissues (one grid, no activation
 * tracking); each tissue's state buffer holds x_s on entry.  Writes x_s .. x_{s+n-1} of tissue
 * e to bufs + e * exp_stride + k * 3 * H * pitch (k = 0 .. n-1); the tissues' state and scratch
 * buffers are overwritten.
 *
 * fk_adjoint_batch_range: fk_adjoint_range for every experiment e, its segment states at
 * bufs + e * exp_stride, its stimuli stimuli[e] (n_stimuli[e] entries).  lam and lam_tmp hold E
 * consecutive states (experiment e at + e * 3 * H * pitch), inj_grads[j] E consecutive states,
 * grad_D E consecutive planes and grad_theta_slots E * fk_adjoint_slots(g) slots.  `workspace`
 * is device memory of fk_adjoint_batch_workspace_bytes(E) bytes (16-byte aligned) that receives
 * the experiments' descriptors. */
size_t fk_adjoint_batch_workspace_bytes(int n_exp);
int fk_batch_recompute(fk_batch *plan, int64_t s, int64_t n, float *bufs, int64_t exp_stride,
                       void *stream);
int fk_adjoint_batch_range(int n_exp, fk_grid g, const float *bufs, int64_t exp_stride, int64_t s,
                           int64_t n, const float *D, const fk_params *p,
                           const fk_stimulus *const *stimuli, const int *n_stimuli, double dt,
                           double dx, float *lam, float *lam_tmp, const int64_t *inj_steps,
                           const float *const *inj_grads, int n_inj, float *grad_D,
                           double *grad_theta_slots, void *workspace, size_t workspace_bytes,
                           void *stream);

#ifdef __cplusplus
}
#endif

#endif /* CARDIAX_GB300_H */
