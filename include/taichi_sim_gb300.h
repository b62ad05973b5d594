/*
 * taichi_sim_gb300 - C ABI of the GB300 (sm_103a) staggered-grid
 * (visco)elastic time stepper.
 *
 * The reference project has no C interface: each backend's
 * ``implementation()`` uploads the host model's tables to a device runtime,
 * runs the per-step kernel loop and reads the results back.  This ABI is
 * that boundary made explicit, with plain pointers and sizes:
 *
 *   ts_create        replaces the buffer uploads of
 *                    sim_taichi_elastic.py:40-132,
 *                    sim_webgpu_viscoelastic.py:57-191 and
 *                    sim_webgpu_3D_viscoelastic.py:62-244
 *   ts_run           replaces the time loops (kernel launches per step)
 *                    sim_taichi_elastic.py:311-335,
 *                    sim_webgpu_viscoelastic.py:469-537,
 *                    sim_webgpu_3D_viscoelastic.py:628-695
 *   ts_status        replaces the per-step velocity-norm read and the
 *                    STABILITY_THRESHOLD test (sim_taichi_elastic.py:320-333,
 *                    sim_webgpu_viscoelastic.py:518-535)
 *   ts_read          replaces the final readbacks
 *                    (sim_taichi_elastic.py:338-339,
 *                    sim_webgpu_viscoelastic.py:540-543,
 *                    sim_webgpu_3D_viscoelastic.py:698-701)
 *   ts_set_sources   replaces the per-shot re-upload of the source term after
 *                    ``set_t0`` (sim_support/simulator.py:329-337)
 *   ts_reset         zeroes the wavefield for the next shot
 *   ts_destroy       releases everything ts_create allocated
 *
 * Every input is a host pointer to the reference's own table, in the
 * reference's layout (C order, last axis fastest); ts_create copies what it
 * needs.  Calls on one handle must not overlap; different handles are
 * independent.  All functions return TS_OK (0) or a positive TS_E* code;
 * ts_strerror gives its text and ts_last_error the detail of the last
 * failure on this thread.
 */
#ifndef TAICHI_SIM_GB300_H
#define TAICHI_SIM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* 2: ts_batch_desc gained the velocity launch shape */
#define TS_ABI_VERSION 2

/* status codes */
#define TS_OK 0
#define TS_E_ARG 1        /* invalid argument or descriptor */
#define TS_E_CUDA 2       /* CUDA runtime error (device lost, launch failure) */
#define TS_E_NOMEM 3      /* device allocation failed */
#define TS_E_NODEV 4      /* no usable sm_103 device */
#define TS_E_STATE 5      /* call not valid in the handle's state */
#define TS_E_TIMEOUT 6    /* a bounded wait between thread blocks gave up (state invalid until ts_reset) */

/* kernel families: which reference backend's semantics to follow */
#define TS_TAICHI2D 0     /* sim_taichi_elastic.py:138-309 (2D elastic); the arithmetic keeps the
                             reference's constants without rounding bias, or with TS_TAICHI_EXACT=1
                             in the environment at ts_create rounds every operation on its own */
#define TS_WGSL2D 1       /* shader_webgpu_viscoelastic.wgsl:829-1141 */
#define TS_WGSL3D 2       /* shader_webgpu_3D_viscoelastic.wgsl:1341-1850 */

/* ts_read targets */
#define TS_VX 0
#define TS_VY 1
#define TS_VZ 2
#define TS_SXX 3
#define TS_SYY 4
#define TS_SZZ 5
#define TS_SXY 6
#define TS_SXZ 7
#define TS_SYZ 8
#define TS_TRACES 9       /* receiver traces, float [n_steps][n_rec] */

typedef struct ts_sim ts_sim;

typedef struct ts_desc {
    int32_t abi_version;       /* TS_ABI_VERSION */
    int32_t family;            /* TS_TAICHI2D / TS_WGSL2D / TS_WGSL3D */
    int32_t nx, ny, nz;        /* full grid incl. CPML and pad; nz = 1 in 2D */
    int32_t n_steps;           /* rows of the source term and of the traces */
    int32_t ord;               /* number of staggered FD coefficients, 1..6 */
    const float *coefs;        /* [ord]  (Simulator._coefs) */
    float dx, dy, dz, dt;      /* grid steps (mm) and time step (us) */
    /* CPML vectors, each of length n_axis - 2 (ord - 1): full-grid a/b/k and
     * half-grid ah/bh/kh per axis (Simulator._a_x, _a_x_half, ...); the z
     * set is unused in 2D and may be NULL. */
    const float *a_x, *b_x, *k_x, *a_xh, *b_xh, *k_xh;
    const float *a_y, *b_y, *k_y, *a_yh, *b_yh, *k_yh;
    const float *a_z, *b_z, *k_z, *a_zh, *b_zh, *k_zh;
    /* material grids [nx][ny][nz]: density as the host model leaves it (the
     * reference averages it in place), P and S velocities */
    const float *rho, *cp, *cs;
    /* attenuation: visco = 0 is the elastic update */
    int32_t visco;
    int32_t n_sls;             /* Zener mechanisms, 1..8 */
    const float *tau;          /* [4][n_sls]: tau_eps_p, tau_sigma_p, tau_eps_s, tau_sigma_s */
    const float *sum_alpha;    /* [2]: sum tau_eps/tau_sigma for P and S */
    /* optional per-cell quality factor (not in the reference): when g_p is
     * non-NULL the memory-variable weight of mechanism l at a cell is
     * zc[l] * g_p[cell] (P) or zc[l] * g_s[cell] (S), with relaxation
     * constants zh[l] = dt / (2 tau_sigma_l) and zm[l] = 1 / (1 + zh[l]). */
    const float *g_p, *g_s;    /* grids, or NULL */
    const float *zc, *zh, *zm; /* [n_sls], or NULL */
    /* sources: the reference's source term and source map */
    const float *source_term;  /* [src_rows][src_cols] (a 1D term is src_cols = 1) */
    int32_t src_rows, src_cols;
    int32_t n_src_el;          /* Simulator._n_src (the WGSL backends' stride) */
    const int32_t *pos_sources;/* grid, column index or -1 */
    /* receivers */
    int32_t n_rec, n_rec_pt;
    const int32_t *pos_sensors;    /* grid, receiver index or -1 (Taichi family) */
    const int32_t *info_rec_pt;    /* [n_rec_pt][dims+1]: grid indices, receiver (WGSL families) */
    const int32_t *offset_sensors; /* [n_rec] first point of each receiver */
    const int32_t *delay_rec;      /* [n_rec] first recorded step */
} ts_desc;

/* Allocate device state for one simulation on the current CUDA device and
 * upload the tables.  The wavefield starts at zero. */
int ts_create(const ts_desc *desc, ts_sim **out);

/* Enqueue n_steps time steps on `stream` (a cudaStream_t, or NULL for the
 * handle's own stream).  Asynchronous; steps past desc->n_steps are
 * rejected with TS_E_ARG. */
int ts_run(ts_sim *sim, int32_t n_steps, void *stream);

/* Wait for queued steps; report the steps done, the largest squared
 * velocity norm seen so far and the first step (0-based) whose norm broke
 * the family's stability threshold (-1 if none).  Any pointer may be NULL. */
int ts_status(ts_sim *sim, int32_t *steps_done, float *max_v2, int32_t *first_unstable_step);

/* Wait for queued steps and copy one field ([nx][ny][nz] floats) or the
 * traces ([n_steps][n_rec] floats) to host memory of `bytes` bytes. */
int ts_read(ts_sim *sim, int32_t what, void *host_dst, size_t bytes);

/* Replace the source term (same shape as at creation), e.g. for a new
 * focal law. */
int ts_set_sources(ts_sim *sim, const float *source_term);

/* Zero the wavefield, memory variables, traces and the step counter. */
int ts_reset(ts_sim *sim);

/* As ts_reset, but enqueued on `stream` (NULL: the handle's own stream)
 * without waiting; later ts_run calls on the same stream see the zeroed
 * state. */
int ts_reset_async(ts_sim *sim, void *stream);

/* Run n_steps steps, the stress update and the velocity update of each
 * step between CUDA events on `stream`, and return their mean device times
 * in milliseconds (ms_per_kernel[2]: stress, velocity; the 3D stress update
 * is two launches).  Advances the simulation like ts_run. */
int ts_profile_steps(ts_sim *sim, int32_t n_steps, void *stream, float *ms_per_kernel);

/* Total kernel launches this handle has issued (graph replays count every
 * kernel node). */
int ts_launch_count(const ts_sim *sim, int64_t *launches);

/* Bytes this handle has copied host->device and device->host so far. */
int ts_transfer_bytes(const ts_sim *sim, int64_t *h2d, int64_t *d2h);

/* Device pointer and size of a field or of the traces, for zero-copy use
 * by a caller on the same device. */
int ts_device_buffer(ts_sim *sim, int32_t what, void **dev_ptr, size_t *pitch_bytes);

/* Enqueue on `stream` (NULL: the handle's own stream) a copy of one field,
 * as it stands after the steps queued so far, to caller memory `dst`
 * (device or pinned host) as [nx][ny][nz] floats with rows dst_pitch bytes
 * apart (0: packed).  Does not wait.  Replaces the reference's live view,
 * which reads the field back every it_display steps
 * (sim_taichi_elastic.py:320-329, sim_webgpu_viscoelastic.py:519-530):
 * the caller records snapshots without a synchronisation per frame. */
int ts_copy_field(ts_sim *sim, int32_t what, void *dst, size_t dst_pitch, void *stream);

/* Number of kernel launches one time step issues (for launch accounting;
 * the persistent path issues its launches per ts_run call instead). */
int ts_launches_per_step(const ts_sim *sim, int32_t *launches);

/* How ts_run advances this handle: TS_PATH_STEPPED, the step's kernels
 * launched once per time step (replayed from a CUDA graph; the default), or
 * TS_PATH_PERSISTENT, every step of the call in one cooperative launch that
 * keeps the wavefield on chip (opt-in with TS_2D_PERSISTENT=1 in the
 * environment at ts_create, for 2D elastic models of order 2 whose row
 * slabs fit shared memory).  Both give the same bits (for family
 * TS_TAICHI2D, with TS_TAICHI_EXACT=1: the persistent kernel rounds every
 * operation on its own, as the stepped path then does). */
#define TS_PATH_STEPPED 0
#define TS_PATH_PERSISTENT 1
int ts_step_path(const ts_sim *sim, int32_t *path);

void ts_destroy(ts_sim *sim);

const char *ts_strerror(int code);
const char *ts_last_error(void);

/*
 * Batched 2D stepping (no single reference counterpart: it replaces the
 * reference's shot loop, Simulator.run() calling implementation() once per
 * emission law, sim_support/simulator.py:326-337, with one device pass over
 * every shot of every phantom).  Each phantom is a full ts_desc (family
 * TS_WGSL2D, ord 2 or 4; all phantoms of a batch share ord, dt, n_steps and
 * the attenuation model) plus n_shots[p] shots; shot s of phantom p injects,
 * at every node of the phantom's source map, column idx of its own table
 * shot_sources[p][s][n_steps][src_cols] (idx = the map's value).  Traces
 * are [n_shots][n_steps][n_rec] per phantom.  block_cells (0 = 8),
 * nodes_per_thread (0 = 2) and shots_per_thread (0 = 1) set the launch
 * shape: blocks of 32 lanes x block_cells nodes along y, each thread
 * updating nodes_per_thread nodes along x for shots_per_thread shots; the
 * velocity launch may take its own block_cells and nodes_per_thread.  They
 * are fixed at creation (order-4 batches take the default shape).
 */
typedef struct ts_batch ts_batch;

typedef struct ts_batch_desc {
    int32_t abi_version;
    int32_t n_phantoms;               /* 1..8 */
    const ts_desc *phantoms;          /* [n_phantoms] */
    const int32_t *n_shots;           /* [n_phantoms] */
    const float *const *shot_sources; /* [n_phantoms] -> [n_shots][n_steps][src_cols] */
    int32_t block_cells;              /* stress launch: nodes along y per block, 0 (= 8), 4 or 8 */
    int32_t nodes_per_thread;         /* stress launch: nodes along x per thread, 0 (= 2), 1, 2 or 4 */
    int32_t shots_per_thread;         /* 0 (= 1), 1 or 2; the shot layout, shared by both launches */
    int32_t velocity_block_cells;     /* velocity launch; 0 = as the stress launch */
    int32_t velocity_nodes_per_thread;/* velocity launch; 0 = as the stress launch */
} ts_batch_desc;

int ts_batch_create(const ts_batch_desc *desc, ts_batch **out);
int ts_batch_run(ts_batch *b, int32_t n_steps, void *stream);
int ts_batch_reset(ts_batch *b, void *stream);
int ts_batch_status(ts_batch *b, int32_t *steps_done, float *max_v2, int32_t *first_unstable_step);
int ts_batch_read_traces(ts_batch *b, int32_t phantom, void *host_dst, size_t bytes);
/* field of every shot of a phantom as [n_shots][nx][ny] floats */
int ts_batch_read_field(ts_batch *b, int32_t phantom, int32_t what, void *host_dst, size_t bytes);
int ts_batch_profile_steps(ts_batch *b, int32_t n_steps, void *stream, float *ms_per_kernel);
int ts_batch_launch_count(const ts_batch *b, int64_t *launches);
/* bytes this batch has copied host->device (creation, sources) and device->host */
int ts_batch_transfer_bytes(const ts_batch *b, int64_t *h2d, int64_t *d2h);
void ts_batch_destroy(ts_batch *b);
const char *ts_batch_last_error(void);

/*
 * Adjoint (time-reversed) gradient of the 2D (visco)elastic stepper, family
 * TS_WGSL2D, ord 2 or 4.  No counterpart in the reference, which has no
 * differentiation: it runs the forward of shader_webgpu_viscoelastic.wgsl:829-1072
 * (receivers :1118-1134) and then the transposed velocity/stress/Zener/CPML
 * updates backward in time.
 *
 * The material enters as the per-node coefficients the stepper uses, on the
 * padded layout [nx][pitch] (ts_adj_pitch; pitch = ny rounded up to 32):
 * L = lambda dt and M = mu dt at the normal node, Ms = mu dt at the shear
 * node, Bx = dt / rho at the vx node, By = dt / rho at the vy node (also the
 * source scale), each a device pointer.  The caller maps per-cell lambda, mu,
 * rho to them with the reference's staggered averaging
 * (shader_webgpu_viscoelastic.wgsl:863-868, 948-950, 1020, 1032) and chains
 * the returned gradients back.  With per-cell Q (desc g_p/g_s) the scales
 * g_p, g_s [nx][pitch] are passed too.
 *
 *   ts_adj_create      checkpoint_every = 0 keeps the 6 per-node features of
 *                      every step (6 * nx * pitch * n_steps floats);
 *                      K > 0 keeps the forward state every K steps and
 *                      recomputes each K-step segment in the backward pass,
 *                      except the trailing segments whose features the
 *                      forward pass records (1 by default)
 *   ts_adj_set_record_segments  number of those trailing segments (memory:
 *                      6 * nx * pitch * K floats each; checkpointed handles)
 *   ts_adj_set_sources replaces the source table (a new shot)
 *   ts_adj_forward     traces[n_steps][n_rec] (device), as ts_run records them
 *   ts_adj_backward    given residual[n_steps][n_rec] = dJ/dtraces (device),
 *                      writes dJ/dL, dJ/dM, dJ/dMs, dJ/dBx, dJ/dBy (device,
 *                      [nx][pitch], overwritten) for the last forward
 *
 * ts_adj_forward and ts_adj_backward are enqueued on `stream` (NULL: the
 * legacy default stream, which is PyTorch's default stream) and do not
 * synchronise; ts_adj_set_sources and ts_adj_read_field synchronise the
 * device.  The handle keeps its own copy of the coefficients of the last
 * forward.
 */
typedef struct ts_adj ts_adj;

typedef struct ts_adj_coefs {
    const float *L, *M, *Ms, *Bx, *By;   /* device, [nx][pitch] */
    const float *g_p, *g_s;              /* device, [nx][pitch]; per-cell Q only */
} ts_adj_coefs;

typedef struct ts_adj_grads {
    float *gL, *gM, *gMs, *gBx, *gBy;    /* device, [nx][pitch] */
} ts_adj_grads;

int ts_adj_create(const ts_desc *desc, int32_t checkpoint_every, ts_adj **out);
int ts_adj_pitch(const ts_adj *a, int32_t *pitch);
int ts_adj_set_record_segments(ts_adj *a, int32_t segments);
int ts_adj_set_sources(ts_adj *a, const float *source_term);   /* host, [src_rows][src_cols] */
int ts_adj_forward(ts_adj *a, const ts_adj_coefs *coefs, float *traces, void *stream);
int ts_adj_backward(ts_adj *a, const float *residual, const ts_adj_grads *grads, void *stream);
/* forward field (TS_VX, TS_VY, TS_SXX, TS_SYY, TS_SXY) after the last
 * ts_adj_forward, as [nx][ny] floats; synchronises the device */
int ts_adj_read_field(ts_adj *a, int32_t what, void *host_dst, size_t bytes);
int ts_adj_launch_count(const ts_adj *a, int64_t *launches);
void ts_adj_destroy(ts_adj *a);
const char *ts_adj_last_error(void);

/*
 * Allocation-free 2D elastic stepper.  No counterpart in the reference: it
 * is for callers that cannot call cudaMalloc (an application that gives
 * this code only buffers from its own pre-sized device pool, a process whose
 * memory budget is fixed at start-up, a time-critical loop that cannot pay
 * an allocation's latency and implicit synchronisation).
 *
 * ts_run_noalloc_2d advances steps step0 .. step0 + n_steps - 1 of a 2D
 * elastic simulation with the WGSL backend's semantics
 * (shader_webgpu_viscoelastic.wgsl:829-1072 with viscoelastic_attn = 0) in
 * device buffers the caller owns, enqueued on `stream` (NULL: the legacy
 * default stream).  Its only scratch, the eight CPML convolution memories
 * (one grid each), lives in a fixed device array of
 * TS_NOALLOC_SCRATCH_FLOATS floats (32 MiB) that every GPU loading this
 * library keeps until exit; grids above TS_NOALLOC_SCRATCH_FLOATS / 8 nodes
 * are rejected with TS_E_ARG.  The function calls no allocating routine.
 * All calls share that array, which keeps the last call's contents: step0 ==
 * 0 clears it (a new simulation); step0 > 0 continues the previous call's
 * simulation.  Calls that overlap on the GPU, or that interleave two
 * simulations, race on it.  The first call on each device looks up the
 * array's device address; make it before any stream capture.  That address
 * is kept for the life of the process and does not survive a reset of the
 * device's context (cudaDeviceReset): do not call this after one.  No
 * stability check is made (the caller can inspect the fields).
 *
 * src_cell and rec_cell are device tables, which the host cannot check: the
 * kernel ignores any entry outside [0, nx * ny).  Several src_cell entries
 * naming the same node all inject (their contributions add up).
 */
#define TS_NOALLOC_SCRATCH_FLOATS (8u << 20)

typedef struct ts_noalloc2d_args {
    int32_t nx, ny;            /* grid, [nx][ny] with y contiguous, no padding */
    int32_t ord;               /* 2..6 */
    float coefs[6];            /* first ord used */
    float dx, dy, dt;
    /* device pointers */
    float *vx, *vy, *sxx, *syy, *sxy;      /* wavefield, read and written */
    const float *rho, *cp, *cs;            /* material grids as the host model leaves them */
    const float *a_x, *b_x, *k_x, *a_xh, *b_xh, *k_xh;   /* [nx - 2 (ord - 1)] */
    const float *a_y, *b_y, *k_y, *a_yh, *b_yh, *k_yh;   /* [ny - 2 (ord - 1)] */
    int32_t n_src;                         /* source nodes */
    const int32_t *src_cell;               /* [n_src] flat node index x * ny + y */
    const float *src_value;                /* [n_rows][n_src] force at each step (divided by rho inside) */
    int32_t n_rec;                         /* receivers, one node each */
    const int32_t *rec_cell;               /* [n_rec] flat node index */
    const int32_t *rec_first_step;         /* [n_rec] first recorded step */
    float *traces;                         /* [n_rows][n_rec], rows < first step left untouched */
    int32_t n_rows;                        /* rows of src_value and traces */
    int32_t step0, n_steps;
} ts_noalloc2d_args;

int ts_run_noalloc_2d(const ts_noalloc2d_args *args, void *stream);
const char *ts_noalloc_last_error(void);

#ifdef __cplusplus
}
#endif
#endif
