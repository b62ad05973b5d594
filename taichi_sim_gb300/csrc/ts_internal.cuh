// Internal device-side layout of the GB300 stepper (not part of the C ABI).
//
// HBM layout, per simulation:
//  * every grid (fields, memory variables, per-cell coefficients) is stored
//    C-order with the last axis padded to a multiple of 32 floats (`pitch`),
//    so each warp row starts on a 128-byte boundary;
//  * CPML convolution memories exist only inside the boundary strips: per
//    axis the strip is a prefix [0, lo) and a suffix [hi, n) of grid
//    indices (where any of the axis' a/b/k tables differs from the identity
//    a = 0, b = 1, k = 1); outside it the reference's update is the identity
//    (psi stays 0 and d/k + psi = d), so it is skipped;
//  * per-cell coefficients are precomputed on the host from rho/cp/cs with
//    the reference's averaging (lambda*dt, mu*dt per stress node, dt/rho per
//    velocity node);
//  * sources are a sparse point list binned by thread block; receivers a
//    CSR list of grid offsets per receiver.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

namespace ts {

constexpr int kMaxOrd = 6;
constexpr int kMaxSls = 8;

// CPML coefficients of one node along one axis: a, b, 1/k and k (the
// Taichi family divides by k, as the reference does).
struct Cpml {
    float a, b, ik, k;
};

// Prefix/suffix strip of one axis: index `i` maps to compact `i` (i < lo)
// or `i - hi + lo` (i >= hi), and is outside the strip otherwise.
struct Strip {
    int lo, hi, width;  // width = lo + (n - hi)
};

__host__ __device__ inline int strip_index(const Strip &s, int i) {
    return i < s.lo ? i : (i >= s.hi ? i - s.hi + s.lo : -1);
}

// Zener constants in update form r' = A r + B d (global taus), or
// r' = A r + (C g) d (per-cell scale g).
struct Zener {
    int n;
    float Ap[kMaxSls], Bp[kMaxSls], As[kMaxSls], Bs[kMaxSls];
};

struct Source {
    int64_t cell;   // flat padded offset
    int col;        // column of the device source table
    float scale;    // rho at the node (stepper), or dt / rho (adjoint forward, batched kernels)
};

// Everything a 2D or 3D kernel reads, passed by value.
// One entry of the 3D coefficient palette: the coefficients each stress
// kernel reads at a node, grouped so that a kernel fetches its own with one
// load.  (The velocity kernel reads its dt / rho pairs from arrays: a
// variant reading them from a second table under the same index measured
// slower, the dependent index load sitting on its critical path.)
struct alignas(16) Pal3 {
    float4 normal;    // lambda dt, mu dt, Q scale p, Q scale s
    float4 shear;     // mu dt at the xy, xz, yz nodes, Q scale s
};

struct StepParams {
    int family;
    int taichi_exact;      // family TS_TAICHI2D: every operation rounded on its own (as the float oracle),
                           // else the unbiased arithmetic (kTaichiU)
    int tx;                // 2D: nodes each thread updates along x (1, 2 or 4)
    int xy_sweep_3d;       // 3D velocity kernel: warps interior in x and y take the x-y sweep
    int stress_pair_3d;    // 3D: normal and shear stress updates in one launch (k_stress3d)
    int snake_3d;          // 3D velocity kernel: x-chunks in reverse launch order
    int prefetch_3d;       // 3D L2 prefetch of a thread's nodes: 2 before the wait (state last written two
                           // launches back), then the rest; 1 the later nodes after the wait; 0 none
    int nx, ny, nz;        // nz = 1 in 2D
    int pitch;             // padded last-axis length (floats)
    int64_t plane;         // ny * pitch (3D x stride); 2D: pitch
    float cd[3][kMaxOrd];  // coef[c] / d_axis (x, y, z)
    // the reference's own factors, for the arithmetic that divides as the
    // reference does (TS_TAICHI2D, and TS_WGSL2D/3D through the stepper):
    // coef[c], 1 / d_axis (float), d_axis, dt
    float coef[kMaxOrd];
    float od[3];
    float odl[3];          // 1 / d_axis - od as a float: od + odl is 1 / d to ~48 bits
    float dd[3];           // the grid steps themselves
    float dt;

    // fields
    float *v[3];           // vx, vy, vz
    float *s[6];           // sxx, syy, szz, sxy, sxz, syz

    // CPML node tables indexed by grid index, full and half grid
    const Cpml *tab_f[3], *tab_h[3];
    Strip strip[3];
    // strip memories: stress kernel psi of velocity derivatives and
    // velocity kernel psi of stress derivatives (see ts_stepper*.cu)
    float *psi[18];

    // per-cell coefficients (the stepper's families: lambda, mu, mu at the
    // shear node(s), rho at the velocity nodes, not folded with dt; the
    // adjoint's forward and the batched kernels: lambda dt, mu dt, dt / rho)
    const float *lam_dt, *mu_dt;          // normal node
    const float *mus_dt[3];               // shear nodes xy, xz, yz (2D: xy)
    const float *dtr[3];                  // rho at the vx, vy nodes (the folded forward: dt / rho; 0: no update)
    const float2 *dtw[3];                 // 3D stepper: dt / rho as a pair (hi, lo), hi + lo exact to ~48 bits
    const float *g_p, *g_s;               // per-cell attenuation scale (or null)
    // 3D coefficient palette (or null): the stress kernels take node i's
    // coefficients from pal[pal_idx[i]] instead of the arrays above
    const uint16_t *pal_idx;
    const Pal3 *pal;
    float *r[6];                          // memory variables, [n_sls] grids each
    int64_t grid_elems;                   // elements of one padded grid
    Zener zen;

    // sources
    const float *src_tab;  // [rows][src_ncol]
    int src_rows, src_ncol;
    const Source *src;     // sorted by block
    const int *src_block_start;  // [n_blocks + 1]

    // receivers
    int n_rec;
    const int *rec_start;  // [n_rec + 1]
    const int64_t *rec_cell;
    const int *rec_first_step;  // record at step k if k >= rec_first_step[s]
    float *traces;              // [rows][n_rec]
    const unsigned char *rec_chunked;  // [n_rec] or null: 1 = summed by k_receiver_chunks, not inline

    // stability bookkeeping
    float v2_threshold;     // a step is unstable when !(v2 <= threshold)
    float *block_max;       // [n_blocks] running max of |v|^2
    int *first_bad;         // min unstable step
    const int *step_base;   // device step counter; step k = *step_base + j

    // 2D adjoint record of one step, [kFeat][grid_elems] (launch_step_2d_feat)
    float *feat;
};

// Receivers with many points, summed after the velocity kernel of every
// step in chunks (ts_receivers.cu).
constexpr int kChunkedMinPoints = 64;   // more points than this: chunked
constexpr int kChunkPoints = 1024;      // points per chunk
struct RecChunks {
    int n_chunks;               // blocks of k_receiver_chunks
    int n_chunked;              // receivers it sums
    const int2 *chunk;          // [n_chunks]: point range [x, y) of the receiver CSR
    const int *receiver;        // [n_chunked]: receiver index
    const int *rchunk;          // [n_chunked + 1]: chunk range of each
    const int64_t *cell;        // the CSR's node offsets
    float *partial;             // [n_chunks]: this step's chunk sums
    unsigned *counter;          // blocks done this step (the last one resets it)
};
void launch_receiver_chunks(const StepParams &p, const RecChunks &rc, int j, cudaStream_t st);

// Arguments of the persistent 2D elastic step kernel (ts_persist2d.cu): the
// regular kernels' parameters plus the exchange buffers between blocks.
struct PersistArgs {
    StepParams p;
    int n_steps;               // steps of this launch, from *p.step_base
    int n_blocks;              // slots of p.block_max
    float *mail;               // [blocks][2 edges][2 step parities][vx, vy][2 ORD - 1 rows][threads]
    unsigned *flags;           // [blocks]: last step whose edge rows are in the mailbox, plus 1
    int *err;                  // [4]: 1 when a wait gave up, its step, its block
    float *samples;            // [rows][n_pts]: syy at each receiver point (CSR position)
    int n_pts;
    const int4 *pts;           // per block: (row in the slab, column, CSR position, 0)
    const int *pts_start;      // [blocks + 1]
    const int4 *srcs;          // per block: (row in the slab, column, table column, dt / rho bits)
    const int *src_start;      // [blocks + 1]
    long long wait_ns;         // bound of every wait on a neighbour
    int stall_block;           // test hook: this block never releases its counter (-1: none)
};

// Persistent path: whether it serves a 2D model (elastic, order 2, a slab of
// rows per block fitting shared memory, every block resident), and its
// shape; and its launch (the kernel, then the receiver sums).
int persist_2d_plan(int family, int ord, int zen_mode, int nx, int ny, int strip_y, int n_sms, int *rows,
                    int *blocks, int *threads, size_t *smem);
cudaError_t launch_persist_2d(const PersistArgs &a, int family, int rows, int blocks, int threads, size_t smem,
                              cudaStream_t st);
// the receiver sums alone: traces of steps [*step_base, *step_base + n_steps) from the samples
cudaError_t launch_persist_2d_receivers(const PersistArgs &a, int n_steps, cudaStream_t st);

// Family TS_TAICHI2D keeps the reference's operation order
// (sim_taichi_elastic.py:152-157, 181-182, 226-229, 263-268, 293-304):
// every product, sum and quotient rounded on its own (the _rn intrinsics are
// never contracted to fma), derivatives as sum of coef * (hi - lo) * (1/d),
// the CPML update as b psi + a d then d / k + psi.  Its results are then the
// bits of a strict IEEE evaluation of the reference's expressions.
__device__ __forceinline__ float taichi_term(float acc, float coef, float hi, float lo, float od) {
    return __fadd_rn(acc, __fmul_rn(__fmul_rn(coef, __fsub_rn(hi, lo)), od));
}
__device__ __forceinline__ float taichi_cpml(float d, float psi_old, float &psi_new, const Cpml &t) {
    psi_new = __fadd_rn(__fmul_rn(t.b, psi_old), __fmul_rn(t.a, d));
    return __fadd_rn(__fdiv_rn(d, t.k), psi_new);
}
// sigma += (lambda div + 2 mu d) dt
__device__ __forceinline__ float taichi_normal(float s, float lam_div, float mu, float d, float dt) {
    return __fadd_rn(s, __fmul_rn(__fadd_rn(lam_div, __fmul_rn(__fmul_rn(2.f, mu), d)), dt));
}
// sigma_xy += (dvx/dy + dvy/dx) mu dt
__device__ __forceinline__ float taichi_shear(float s, float e, float mu, float dt) {
    return __fadd_rn(s, __fmul_rn(__fmul_rn(e, mu), dt));
}
// v += src + f dt / rho (src: the source's force dt / rho, or 0); no update where rho <= 0
__device__ __forceinline__ float taichi_velocity(float v, float f, float src, float rho, float dt) {
    return rho > 0.f ? __fadd_rn(v, __fadd_rn(src, __fdiv_rn(__fmul_rn(f, dt), rho))) : v;
}

// x / b without a division instruction, rounded as the division almost
// always is (Markstein's correction step with r = RN(1/b)): q = x r,
// e = x - q b exactly (fma), q + e r.
__device__ __forceinline__ float qdiv(float x, float b, float r) {
    const float q = x * r;
    const float e = fmaf(-q, b, x);
    return fmaf(e, r, q);
}
// WGSL velocity update v + (f dt) / rho (shader_webgpu_viscoelastic.wgsl:
// 1020-1024, 1049-1052) with w = dt / rho given as a pair (hi, lo) whose sum
// holds it to ~48 bits (0 where rho <= 0: no update): the only roundings are
// those of the two fmas, none repeating at every node
__device__ __forceinline__ float wgsl_velocity(float v, float f, float2 w) { return fmaf(f, w.x, fmaf(f, w.y, v)); }
// the same update from rho itself, f dt divided by rho (one correction step
// on a correctly rounded reciprocal); no update where rho <= 0.  Fewer bytes
// than the pair (the 2D kernels, whose working set is L2-resident, measured
// faster with it; the 3D ones slower).
__device__ __forceinline__ float wgsl_velocity_rho(float v, float f, float rho, float dt) {
    return rho > 0.f ? v + qdiv(f * dt, rho, __frcp_rn(rho)) : v;
}
// s / d for a grid step d with 1 / d = od + odl (to ~48 bits): unbiased
__device__ __forceinline__ float dscale(float s, float od, float odl) { return fmaf(s, od, s * odl); }
// WGSL source force src dt / rho (wgsl:1059-1065)
__device__ __forceinline__ float wgsl_source(float src, float rho, float dt) {
    return qdiv(src * dt, rho, __frcp_rn(rho));
}

// Slots of the 2D adjoint record: what the stress and velocity updates
// multiply lambda*dt, mu*dt (normal node: x and y rows), mu*dt (shear node)
// and dt/rho (vx, vy nodes) by.
enum { kFeatLam = 0, kFeatMuX, kFeatMuY, kFeatShear, kFeatVx, kFeatVy, kFeat };

// Programmatic dependent launch: a step kernel may be scheduled while the
// previous kernel of the stream drains.  Before the wait it may only read
// data no earlier kernel writes (coefficients, tables); after it, all
// writes of the previous kernels are visible to coherent loads.  Fields an
// earlier kernel wrote are never read through the non-coherent (read-only)
// path: that kernel's lifetime overlaps this one's, and such reads returned
// stale values in a few percent of runs.  The trigger lets the next
// kernel's launch start once every block of this one has issued it.
// Hint: bring the 128-byte line holding `a` into L2 (no register, no wait).
__device__ __forceinline__ void prefetch_l2(const void *a) { asm volatile("prefetch.global.L2 [%0];" ::"l"(a)); }

__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// Stability bookkeeping of one warp: max |v|^2 into the block's slot and the
// first unstable step, both as reductions the warp does not wait for.
__device__ __forceinline__ void warp_stability(float v2, bool bad, unsigned *block_slot, int *first_bad, int k) {
    const unsigned m = __reduce_max_sync(0xffffffffu, __float_as_uint(v2));
    const unsigned any_bad = __ballot_sync(0xffffffffu, bad);
    if ((threadIdx.x & 31) == 0) {
        atomicMax(block_slot, m);
        if (any_bad) atomicMin(first_bad, k);
    }
}

// Launch a step kernel with programmatic stream serialisation (see above).
template <typename... Params, typename... Args>
inline void launch_pdl(void (*kern)(Params...), dim3 grid, dim3 block, cudaStream_t st, Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, kern, args...);
}

// Launch helpers (defined per dimension).  `parts` selects the kernels of
// one step: 1 = stress, 2 = velocity, 3 = both (in that order).
void launch_step_2d(const StepParams &p, int ord, int zen_mode, int j, cudaStream_t st, int parts = 3);
// Family TS_WGSL2D step with coefficients folded with dt (the adjoint's
// forward; p.tx 1 or 2 at order 2, 2 above; folded: ord 2 or 4), without and
// with the adjoint record written to p.feat.
void launch_step_2d_folded(const StepParams &p, int ord, int zen_mode, int j, cudaStream_t st);
void launch_step_2d_feat(const StepParams &p, int ord, int zen_mode, int j, cudaStream_t st);
void launch_step_3d(const StepParams &p, int ord, int zen_mode, int j, cudaStream_t st, int parts = 3);
// the palette instantiations of the stress kernels (p.pal set; 32-bit offsets)
void launch_step_3d_pal(const StepParams &p, int ord, int zen_mode, int j, cudaStream_t st, int parts);
// the array instantiations of orders 3 to 6 (ts_stepper3d_o<N>.cu)
void launch_step_3d_arrays_3(const StepParams &p, int zen_mode, int j, cudaStream_t st, int parts);
void launch_step_3d_arrays_4(const StepParams &p, int zen_mode, int j, cudaStream_t st, int parts);
void launch_step_3d_arrays_5(const StepParams &p, int zen_mode, int j, cudaStream_t st, int parts);
void launch_step_3d_arrays_6(const StepParams &p, int zen_mode, int j, cudaStream_t st, int parts);
void launch_reset_scalars(int *first_bad, int *step_base, cudaStream_t st);
void launch_advance(int *step_base, int n, cudaStream_t st);
int blocks_2d(const StepParams &p);
int blocks_3d(const StepParams &p);
constexpr int kBX2 = 32, kBY2 = 8;              // 2D block: 32 (y) x 8 (x) threads, p.tx nodes each along x

// Flat index of the 2D block that updates node (x, y).
inline int block_of_2d(const StepParams &p, int x, int y) {
    const int gx = (p.ny + kBX2 - 1) / kBX2;
    return (x / (kBY2 * p.tx)) * gx + y / kBX2;
}
// 2D nodes per thread along x: one up to 768^2 grids (the L2-resident
// small grids want more warps in flight), two from 1024^2 (fewer index and
// bookkeeping instructions per node); TS_2D_NODES_PER_THREAD = 1, 2 or 4
// overrides it.  Measured: elastic 512^2 26.7 against 22.6 Gcell/s,
// viscoelastic 640^2 33.9 / 32.1, 768^2 38.6 / 38.2, 1024^2 43.6 / 47.4.
int nodes_per_thread_2d(int64_t cells);

// 3D kernels: blocks of 32 (z) x 8 (y) threads, each updating kTX3S (stress
// kernels) or p.tx (velocity kernel: 4 for order 2, 2 above, where 4 spills)
// consecutive nodes along x (measured on the 256^3 three-mechanism case
// against 1, 2 and 4).
#ifndef TS_STRESS3D_TX
#define TS_STRESS3D_TX 4
#endif
constexpr int kBX3 = 32, kBY3 = 8, kTX3S = TS_STRESS3D_TX;
// The 8 warps of a block cover kZW3 consecutive 32-node runs along z (the
// contiguous axis) times 8 / kZW3 rows along y (2 measured best of 1, 2, 4,
// 8 on the 256^3 case: longer contiguous runs per block, y-neighbours still
// shared in L1).
#ifndef TS_3D_Z_RUNS
#define TS_3D_Z_RUNS 2
#endif
constexpr int kZW3 = TS_3D_Z_RUNS, kZB3 = kBX3 * kZW3, kYB3 = kBY3 / kZW3;
#ifndef TS_VELOCITY3D_TX
#define TS_VELOCITY3D_TX 4
#endif
constexpr int velocity_tx_3d(int ord) { return ord == 2 ? TS_VELOCITY3D_TX : 2; }

// Flat index of the 3D velocity block that updates node (x, y, z).
inline int block_of_3d(const StepParams &p, int x, int y, int z) {
    const int gx = (p.nz + kZB3 - 1) / kZB3, gy = (p.ny + kYB3 - 1) / kYB3, nch = (p.nx + p.tx - 1) / p.tx;
    const int bz = p.snake_3d ? nch - 1 - x / p.tx : x / p.tx;   // launch order of the x-chunk
    return (bz * gy + y / kYB3) * gx + z / kZB3;
}

}  // namespace ts
