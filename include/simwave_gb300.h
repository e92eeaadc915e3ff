/*
 * simwave_gb300.h -- C ABI of libsimwave_gb300.so, the GB300 (sm_103a)
 * implementation of simwave's forward time-stepping operator.
 *
 * Two families of entry points:
 *
 * 1. Host-pointer drop-ins, one per (dimension, density, precision). Each has
 *    exactly the argument list of the reference's `forward` C function for
 *    that variant, as marshalled by the reference's Middleware with ctypes
 *    (simwave/kernel/backend/middleware.py:107-204): numpy arrays arrive as
 *    pointers, Python ints as size_t, float32/float64 scalars as float/double.
 *    `u` (num_snapshots wavefield slots) and `receivers` (end_timestep x
 *    num_receivers) are in/out host buffers; all other arrays are read-only.
 *    The return value is the call's wall time in seconds, as in the
 *    reference; a negative value is an error status (see SIMWAVE_E_*), with a
 *    message from simwave_last_error(). The library never exits the process.
 *
 * 2. A device-pointer entry (simwave_forward_device) that runs the same
 *    operator on arrays already resident on the GPU, ordered on a caller's
 *    CUDA stream, with an explicit row pitch for the fastest grid axis.
 *
 * Grid layout: C order of the extended grid (model + damping layer + halo),
 * z slowest; 2D arrays are (nz, nx), 3D arrays are (nz, nx, ny).
 * Boundary codes: 0 none, 1 null Dirichlet, 2 null Neumann, ordered
 * (z_before, z_after, x_before, x_after[, y_before, y_after]).
 *
 * Difference from the reference, by design: the 3D variable-density x-axis
 * first derivatives use the layout's row stride ny; the reference uses nx
 * (variable_density/3d/wave.c:185-186). Results agree whenever nx == ny.
 */
#ifndef SIMWAVE_GB300_H
#define SIMWAVE_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* error statuses (returned negated as double by the host entries) */
#define SIMWAVE_OK 0
#define SIMWAVE_E_ARGUMENT 1   /* invalid argument or unsupported size */
#define SIMWAVE_E_SCHEDULE 2   /* time range / stride needs more slots */
#define SIMWAVE_E_CUDA 3       /* CUDA runtime or launch error */
#define SIMWAVE_E_MEMORY 4     /* device allocation failed */
#define SIMWAVE_E_TIMEOUT 5    /* a bounded device wait gave up */

/* ---- host-pointer drop-ins ------------------------------------------------
 * replaces: forward() in
 *   simwave/kernel/backend/c_code/forward/constant_density/2d/wave.c:23-36 */
double simwave_forward_2d_cd_f32(
    float *u, float *velocity, float *damp, float *wavelet,
    size_t wavelet_size, size_t wavelet_count, float *coeff,
    size_t *boundary_conditions, size_t *src_points_interval,
    size_t src_points_interval_size, float *src_points_values,
    size_t src_points_values_size, size_t *src_points_values_offset,
    size_t *rec_points_interval, size_t rec_points_interval_size,
    float *rec_points_values, size_t rec_points_values_size,
    size_t *rec_points_values_offset, float *receivers, size_t num_sources,
    size_t num_receivers, size_t nz, size_t nx, float dz, float dx,
    size_t saving_stride, float dt, size_t begin_timestep,
    size_t end_timestep, size_t space_order, size_t num_snapshots);

/* same, built with -DDOUBLE (wave.c:17-21) */
double simwave_forward_2d_cd_f64(
    double *u, double *velocity, double *damp, double *wavelet,
    size_t wavelet_size, size_t wavelet_count, double *coeff,
    size_t *boundary_conditions, size_t *src_points_interval,
    size_t src_points_interval_size, double *src_points_values,
    size_t src_points_values_size, size_t *src_points_values_offset,
    size_t *rec_points_interval, size_t rec_points_interval_size,
    double *rec_points_values, size_t rec_points_values_size,
    size_t *rec_points_values_offset, double *receivers, size_t num_sources,
    size_t num_receivers, size_t nz, size_t nx, double dz, double dx,
    size_t saving_stride, double dt, size_t begin_timestep,
    size_t end_timestep, size_t space_order, size_t num_snapshots);

/* replaces: forward() in
 *   simwave/kernel/backend/c_code/forward/variable_density/2d/wave.c:23-36 */
double simwave_forward_2d_vd_f32(
    float *u, float *velocity, float *density, float *damp, float *wavelet,
    size_t wavelet_size, size_t wavelet_count, float *coeff_order2,
    float *coeff_order1, size_t *boundary_conditions,
    size_t *src_points_interval, size_t src_points_interval_size,
    float *src_points_values, size_t src_points_values_size,
    size_t *src_points_values_offset, size_t *rec_points_interval,
    size_t rec_points_interval_size, float *rec_points_values,
    size_t rec_points_values_size, size_t *rec_points_values_offset,
    float *receivers, size_t num_sources, size_t num_receivers, size_t nz,
    size_t nx, float dz, float dx, size_t saving_stride, float dt,
    size_t begin_timestep, size_t end_timestep, size_t space_order,
    size_t num_snapshots);

double simwave_forward_2d_vd_f64(
    double *u, double *velocity, double *density, double *damp,
    double *wavelet, size_t wavelet_size, size_t wavelet_count,
    double *coeff_order2, double *coeff_order1, size_t *boundary_conditions,
    size_t *src_points_interval, size_t src_points_interval_size,
    double *src_points_values, size_t src_points_values_size,
    size_t *src_points_values_offset, size_t *rec_points_interval,
    size_t rec_points_interval_size, double *rec_points_values,
    size_t rec_points_values_size, size_t *rec_points_values_offset,
    double *receivers, size_t num_sources, size_t num_receivers, size_t nz,
    size_t nx, double dz, double dx, size_t saving_stride, double dt,
    size_t begin_timestep, size_t end_timestep, size_t space_order,
    size_t num_snapshots);

/* replaces: forward() in
 *   simwave/kernel/backend/c_code/forward/constant_density/3d/wave.c:23-36 */
double simwave_forward_3d_cd_f32(
    float *u, float *velocity, float *damp, float *wavelet,
    size_t wavelet_size, size_t wavelet_count, float *coeff,
    size_t *boundary_conditions, size_t *src_points_interval,
    size_t src_points_interval_size, float *src_points_values,
    size_t src_points_values_size, size_t *src_points_values_offset,
    size_t *rec_points_interval, size_t rec_points_interval_size,
    float *rec_points_values, size_t rec_points_values_size,
    size_t *rec_points_values_offset, float *receivers, size_t num_sources,
    size_t num_receivers, size_t nz, size_t nx, size_t ny, float dz,
    float dx, float dy, size_t saving_stride, float dt,
    size_t begin_timestep, size_t end_timestep, size_t space_order,
    size_t num_snapshots);

double simwave_forward_3d_cd_f64(
    double *u, double *velocity, double *damp, double *wavelet,
    size_t wavelet_size, size_t wavelet_count, double *coeff,
    size_t *boundary_conditions, size_t *src_points_interval,
    size_t src_points_interval_size, double *src_points_values,
    size_t src_points_values_size, size_t *src_points_values_offset,
    size_t *rec_points_interval, size_t rec_points_interval_size,
    double *rec_points_values, size_t rec_points_values_size,
    size_t *rec_points_values_offset, double *receivers, size_t num_sources,
    size_t num_receivers, size_t nz, size_t nx, size_t ny, double dz,
    double dx, double dy, size_t saving_stride, double dt,
    size_t begin_timestep, size_t end_timestep, size_t space_order,
    size_t num_snapshots);

/* replaces: forward() in
 *   simwave/kernel/backend/c_code/forward/variable_density/3d/wave.c:23-36 */
double simwave_forward_3d_vd_f32(
    float *u, float *velocity, float *density, float *damp, float *wavelet,
    size_t wavelet_size, size_t wavelet_count, float *coeff_order2,
    float *coeff_order1, size_t *boundary_conditions,
    size_t *src_points_interval, size_t src_points_interval_size,
    float *src_points_values, size_t src_points_values_size,
    size_t *src_points_values_offset, size_t *rec_points_interval,
    size_t rec_points_interval_size, float *rec_points_values,
    size_t rec_points_values_size, size_t *rec_points_values_offset,
    float *receivers, size_t num_sources, size_t num_receivers, size_t nz,
    size_t nx, size_t ny, float dz, float dx, float dy,
    size_t saving_stride, float dt, size_t begin_timestep,
    size_t end_timestep, size_t space_order, size_t num_snapshots);

double simwave_forward_3d_vd_f64(
    double *u, double *velocity, double *density, double *damp,
    double *wavelet, size_t wavelet_size, size_t wavelet_count,
    double *coeff_order2, double *coeff_order1, size_t *boundary_conditions,
    size_t *src_points_interval, size_t src_points_interval_size,
    double *src_points_values, size_t src_points_values_size,
    size_t *src_points_values_offset, size_t *rec_points_interval,
    size_t rec_points_interval_size, double *rec_points_values,
    size_t rec_points_values_size, size_t *rec_points_values_offset,
    double *receivers, size_t num_sources, size_t num_receivers, size_t nz,
    size_t nx, size_t ny, double dz, double dx, double dy,
    size_t saving_stride, double dt, size_t begin_timestep,
    size_t end_timestep, size_t space_order, size_t num_snapshots);

/* Message of the calling thread's last failed call ("" if none).
 * No reference counterpart: the reference has no error path
 * (C) or exits the process (cuda/wave.cu:16-24). */
const char *simwave_last_error(void);

/* ---- device-pointer entry ---------------------------------------------- */

/* One forward problem on device-resident arrays. Field names follow the
 * reference's `forward` arguments (middleware.py:160-204). All pointers
 * marked (device) are GPU addresses; coefficients and boundary codes are read
 * from host memory during the call.
 *
 * Grid arrays (u slots, velocity, density, damp) share one layout: point
 * (i, j[, k]) of the fastest axis index f = x (2D) or y (3D) lives at
 *   2D: i * pitch + lead + j
 *   3D: (i * nx + j) * pitch + lead + k
 * elements from the array base, and consecutive u slots are slot_stride
 * elements apart. pitch >= lead + fastest extent. A dense array has
 * pitch = fastest extent and lead = 0. */
typedef struct simwave_problem {
    int dim;                  /* 2 or 3 */
    int variable_density;     /* 0 constant, 1 variable */
    int precision;            /* 4 (float32) or 8 (float64) */
    int space_order;          /* even, 2..20 */
    size_t nz, nx, ny;        /* extended shape; ny = 1 in 2D */
    size_t pitch, lead, slot_stride;
    double dz, dx, dy, dt;
    void *u;                  /* (device) num_snapshots slots, in/out */
    size_t num_snapshots;
    const void *velocity;     /* (device) */
    const void *density;      /* (device) NULL for constant density */
    const void *damp;         /* (device) */
    const void *wavelet;      /* (device) wavelet_size * wavelet_count */
    size_t wavelet_size, wavelet_count;
    const void *coeff_order2; /* (host) space_order/2 + 1 values */
    const void *coeff_order1; /* (host) idem, variable density only */
    const size_t *boundary_conditions;      /* (host) 2*dim codes */
    const size_t *src_points_interval;      /* (device) 2*dim per source */
    const void *src_points_values;          /* (device) */
    const size_t *src_points_values_offset; /* (device) num_sources + 1 */
    size_t src_points_values_size;
    size_t num_sources;
    const size_t *rec_points_interval;      /* (device) */
    const void *rec_points_values;          /* (device) */
    const size_t *rec_points_values_offset; /* (device) */
    size_t rec_points_values_size;
    size_t num_receivers;
    void *receivers;          /* (device) end_timestep * num_receivers, out */
    size_t saving_stride, begin_timestep, end_timestep;
    unsigned flags;           /* SIMWAVE_FLAG_* */
} simwave_problem;

/* flags */
#define SIMWAVE_FLAG_TIME_KERNELS 1u  /* time the stencil launches (events) */
#define SIMWAVE_FLAG_WINDOWS_CHECKED 2u /* caller validated the KWS windows
                                          (intervals inside the grid, offsets
                                          consistent); skips the device->host
                                          copy the library otherwise makes to
                                          check them */

#define SIMWAVE_FLAG_GENERIC_KERNEL 4u  /* force the one-thread-per-point
                                           stencil (testing and comparison) */
#define SIMWAVE_FLAG_STEP_LAUNCHES 8u   /* 2D float32: launch each step's
                                           kernels separately even where the
                                           whole run would go in one persistent
                                           launch (grids up to 1.5 M interior
                                           points) -- testing and timing */

/* Preferred layout of the fastest axis for a grid of `fastest_extent`
 * points at `space_order` and `precision` bytes: writes the row pitch and
 * leading offset (elements) that align each row's first interior point to
 * 128 bytes. Returns SIMWAVE_OK or SIMWAVE_E_ARGUMENT.
 * No reference counterpart (the reference uses dense arrays). */
int simwave_layout(size_t fastest_extent, int space_order, int precision,
                   size_t *pitch, size_t *lead);

/* Run the forward loop on `stream` (a cudaStream_t, NULL = default stream).
 * Returns SIMWAVE_OK or an error status; the work is stream-ordered and the
 * call returns before it completes unless SIMWAVE_FLAG_TIME_KERNELS is set
 * (then it synchronises the stream to read the timers).
 * No reference counterpart: the reference allocates and copies per call. */
int simwave_forward_device(const simwave_problem *problem, void *stream);

/* Stencil kernel selection for the float32 3D path (process-wide).
 * AUTO picks per order and density; the others force one variant (tuning
 * and tests). Returns SIMWAVE_OK or SIMWAVE_E_ARGUMENT.
 * No reference counterpart. */
#define SIMWAVE_POLICY_AUTO 0
#define SIMWAVE_POLICY_SCALAR_TILED 1   /* one y point per thread */
#define SIMWAVE_POLICY_VEC_2CTA 2       /* float4 along y, 2 CTAs per SM */
#define SIMWAVE_POLICY_VEC_1CTA 3       /* float4 along y, 1 CTA per SM */
#define SIMWAVE_POLICY_VEC_SMEMQ 4      /* float4 along y, density z-queue in
                                           shared memory, 2 CTAs per SM */
#define SIMWAVE_POLICY_VEC_2CTA_ROT 5   /* float4, register queues rotated by
                                           unrolling, 2 CTAs per SM */
#define SIMWAVE_POLICY_VEC_1CTA_ROT 6   /* same, 1 CTA per SM */
#define SIMWAVE_POLICY_VEC_PACKED 7     /* float4 along y with packed f32x2
                                           arithmetic, density z-queue in shared
                                           memory, 2 CTAs per SM */
#define SIMWAVE_POLICY_VEC_PACKED_1CTA 8 /* same, 1 CTA per SM */
#define SIMWAVE_POLICY_TMEM 9           /* orders <= 8: packed arithmetic, the
                                           u and density z queues in tensor
                                           memory, damping from per-axis
                                           tables; 8 x rows per CTA, 2 CTAs
                                           per SM */
#define SIMWAVE_POLICY_STAGE_RELEASE 10 /* orders <= 8: packed arithmetic, u
                                           queue in registers, density z term
                                           from a per-run grid, 12 x rows per
                                           CTA, 1 CTA per SM, six planes in
                                           flight refilled by the last warp to
                                           finish each (no CTA barrier per
                                           plane); AUTO for order 8 with
                                           variable density */
int simwave_set_kernel_policy(int policy);

/* How the host-pointer entries move grids (process-wide).
 * AUTO: page-lock the caller's grids (and the record's rows) for the
 *   duration of the call, then copy as STAGED, asynchronously (STAGED
 *   from pageable memory if locking fails); STAGED: one contiguous copy per
 *   grid through a dense device staging buffer, repacked on the device
 *   into or out of the pitched layout; DIRECT: kernels read and write
 *   the caller's pageable arrays (devices with pageable-memory access only,
 *   else STAGED). Grid snapshots leave while the time loop is still running.
 * No reference counterpart. */
#define SIMWAVE_TRANSFER_AUTO 0
#define SIMWAVE_TRANSFER_STAGED 1
#define SIMWAVE_TRANSFER_DIRECT 2
int simwave_set_transfer_mode(int mode);

/* Wait for `stream` and report device-side failures of the forward calls
 * enqueued on it (a bounded wait that expired: SIMWAVE_E_TIMEOUT). Clears
 * the recorded status. No reference counterpart. */
int simwave_device_status(void *stream);

/* ---- allocation-free variant -------------------------------------------
 * simwave_forward_device_noalloc runs the same float32 3D forward as
 * simwave_forward_device on caller-owned device arrays, but allocates no
 * device memory at all: no cudaMalloc, cudaFree or allocating library call.
 * It exists for callers that cannot let us allocate while they run: a host
 * framework that owns the device memory budget through its own pool, or a
 * serving loop in which an allocation would synchronise the device and stall
 * unrelated work. Its scratch (two per-point coefficient grids and 256 bytes
 * of status words) lives in one file-scope device array of
 * SIMWAVE_NOALLOC_SCRATCH_BYTES that every GPU loading this library keeps
 * until the process exits. Limits: 3D float32 problems only; a grid of at
 * most (SIMWAVE_NOALLOC_SCRATCH_BYTES - 256) / 8 pitched points (larger grids
 * are refused with SIMWAVE_E_ARGUMENT and a simwave_last_error() message);
 * of the flags only SIMWAVE_FLAG_WINDOWS_CHECKED (any other flag is
 * refused); the layout must suit the tiled kernel (the one simwave_layout()
 * returns does). The call reads results back to the host and waits for
 * `stream` mid-call, so it must not be made on a stream that is being
 * captured into a CUDA graph: such a stream is refused with
 * SIMWAVE_E_ARGUMENT before any work is enqueued. The first call on a device
 * looks up the array's device address (with that device current). All calls
 * share the one array and its status words are reset at the start of each
 * call: calls that overlap on the GPU race on it and must be serialised.
 * No reference counterpart. */
#define SIMWAVE_NOALLOC_SCRATCH_BYTES (32u << 20)
int simwave_forward_device_noalloc(const simwave_problem *problem, void *stream);

/* ---- batch engine: many 2D shots advanced together ------------------------
 * Shots are 2D float32 problems on device-resident arrays (pitched layout of
 * simwave_layout(), KWS windows already validated: SIMWAVE_FLAG_WINDOWS_CHECKED);
 * the arrays must stay valid until the shot is released. Each step of the
 * batch advances every unfinished shot by one time step with one launch per
 * (order, density) group for the stencil and one per sparse term for all
 * shots; the launch sequence of 16 steps is captured once as a CUDA graph and
 * replayed while the shot set is unchanged. Results equal the single-shot
 * entries' (same operator and schedule).
 * No reference counterpart (the reference runs one shot per call). */
typedef struct simwave_batch simwave_batch;
int simwave_batch_create(simwave_batch **out);
int simwave_batch_destroy(simwave_batch *batch);
/* Add a shot (problem fields as for simwave_forward_device); writes its id. */
int simwave_batch_add(simwave_batch *batch, const simwave_problem *problem,
                      int *shot_id);
/* Advance every unfinished shot by up to `steps` time steps, ordered after
 * prior work on `stream`; `stream` waits for the batch. */
int simwave_batch_run(simwave_batch *batch, int steps, void *stream);
/* Time steps left for a shot (0 when finished). */
int simwave_batch_remaining(simwave_batch *batch, int shot_id, int *steps);
/* Remove a shot; a finished shot's slots are put back in the reference's
 * order first. Waits for the batch's work. An unfinished shot leaves its
 * latest two levels in the schedule's current slots (a later call can
 * resume from there); with time blocking, the third rotating slot may hold
 * an older level than the per-step kernels would have left in it. */
int simwave_batch_release(simwave_batch *batch, int shot_id);
/* Tuning: stencil tile height for one space order: 8, 16 or 32 rows staged
 * at once (with an R-row halo each), or 64, 128 or 256 rows streamed
 * through a ring of 64 staged rows (each row staged once per tile). */
int simwave_batch_set_tile_rows(simwave_batch *batch, int space_order, int rows);
/* Tuning: time-blocking depth for one space order -- 1 (default: a launch
 * per step), or 2..4 steps per launch where depth x space_order / 2 <= 36
 * (the tile keeps >= 32 owned rows) and the tile keeps >= 64 owned
 * columns. A tile stages 104 rows of u_cur, u_prev, C and Q once and
 * advances them `depth` steps in shared memory (sources, boundary
 * conditions and receiver records included), trading recomputed tile
 * margins for fewer passes over HBM. Shots with variable density or a
 * source window reaching into the halo keep depth 1. Results equal depth
 * 1's bit for bit (receiver windows are copied per tile and summed in the
 * per-step order). */
int simwave_batch_set_depth(simwave_batch *batch, int space_order, int depth);
/* Depth a shot runs at under the current settings. */
int simwave_batch_depth(simwave_batch *batch, int shot_id, int *depth);
/* Kernel launches enqueued so far (graph nodes counted per replay). */
int simwave_batch_launches(simwave_batch *batch, size_t *launches);

/* Statistics of the calling thread's last successful forward call. */
typedef struct simwave_stats {
    double seconds;           /* wall time of the call */
    double stencil_ms;        /* summed stencil kernel time (if timed) */
    double updates;           /* interior point updates performed */
    size_t stencil_launches;  /* stencil kernel launches */
    size_t kernel_launches;   /* all kernel launches of this library */
    size_t h2d_bytes, d2h_bytes;
    int stencil_variant;      /* 0 generic, 1 tiled, 2 tiled 2D, all steps
                                 in one persistent launch, 3 tiled 2D, each
                                 step (stencil, sources, boundaries,
                                 receivers) in one launch */
    int stencil_kernel;       /* 3D float32 tiled runs: the SIMWAVE_POLICY_*
                                 of the stencil kernel launched (AUTO
                                 resolved); 0 otherwise */
} simwave_stats;

/* No reference counterpart (the reference returns only its wall time). */
int simwave_last_stats(simwave_stats *out);

/* ---- velocity gradient (2D, float32, constant or variable density) ------
 * No reference counterpart: the reference offers only the forward operator
 * (simwave/kernel/backend/compiler.py:128-130) and its middleware dispatches
 * only 'forward' (simwave/kernel/backend/middleware.py:103-105).
 *
 * The gradient is that of J = sum(g * receivers) with respect to the
 * velocity grid, for a cotangent g of the shot record, through the exact
 * discrete forward loop (damping, KWS source and receiver windows, boundary
 * conditions), with dt, the damping mask, the density and the windows held
 * fixed. Variable density needs the tiled layout of simwave_layout()
 * (SIMWAVE_E_ARGUMENT otherwise). The
 * forward starts from zero levels; `u`, `num_snapshots`, `saving_stride` and
 * `slot_stride` are not used. KWS windows must lie inside the interior
 * (SIMWAVE_E_ARGUMENT otherwise), and each interior extent must be at least
 * space_order + 2. All work is ordered on `stream`; the calls copy the KWS
 * windows to the host (a stream synchronisation) and allocate their scratch
 * on the stream (cudaMallocAsync). */

/* Number of grids (nz * pitch float32 elements each) the checkpoint buffer
 * of a run with checkpoint `interval` steps needs: 2 * ceil(steps / interval). */
int simwave_gradient_checkpoints(const simwave_problem *problem, size_t interval,
                                 size_t *grids);

/* Forward pass: writes the shot record into `receivers` (row n-1 from level
 * n, as simwave_forward_device) and the level pair (u^(n-1), u^n) before
 * every `interval`-th step into `checkpoints` (device). */
int simwave_gradient_forward(const simwave_problem *problem, size_t interval,
                             void *checkpoints, void *stream);

/* Reverse pass: from the checkpoints of simwave_gradient_forward (same
 * problem and interval) and `grad_receivers` (device, end_timestep rows of
 * num_receivers float32), writes dJ/dv into `grad_velocity` (device, one
 * grid in the problem's pitched layout; zero outside the interior). Needs
 * (interval + 8) grids of scratch (+ 2 with variable density), plus
 * interval rows of the Dirichlet lines when an edge is null_dirichlet. */
int simwave_gradient_backward(const simwave_problem *problem, size_t interval,
                              const void *checkpoints, const void *grad_receivers,
                              void *grad_velocity, void *stream);

/* Several shots of one inversion at once: `nshots` problems (an array of
 * structs) of one layout, space order, density kind and step range, with a
 * checkpoint buffer each (simwave_gradient_checkpoints grids each). The
 * forward writes every shot's record and checkpoints; the reverse pass
 * writes into `grad_velocity` the SUM over the shots of dJ_s/dv for the
 * cotangents grad_receivers[s]. When every shot takes the one-launch step
 * (the first and last 16-row and 128-column tiles hold r + 1 rows and
 * columns, after the tiling offset) the shots advance in lockstep, one
 * launch per step for all of them; otherwise one after another. The reverse
 * pass keeps every shot's segment levels at once: (interval + 8) grids a
 * shot. No reference counterpart. */
int simwave_gradient_forward_shots(const simwave_problem *problems, size_t nshots,
                                   size_t interval, void *const *checkpoints, void *stream);
int simwave_gradient_backward_shots(const simwave_problem *problems, size_t nshots,
                                    size_t interval, const void *const *checkpoints,
                                    const void *const *grad_receivers, void *grad_velocity,
                                    void *stream);

#ifdef __cplusplus
}
#endif

#endif /* SIMWAVE_GB300_H */
