// Persistent 2D elastic stepper: many time steps in one cooperative launch,
// the wavefield held on chip between steps.
//
// A 512^2 elastic state is ~15 MB; the two-launch step (ts_kernels2d.cuh)
// then spends most of its time launching and draining grid-wide kernels,
// not moving bytes.  Here each thread block owns a slab of R consecutive
// rows (x) times every column (y), one column per thread, and keeps in
// shared memory what its step needs: the velocities on its rows plus
// NH = 2 ORD - 1 rows on each side, the stresses on its rows plus ORD rows on
// each side, the CPML memories of those rows; the per-node coefficients sit
// in registers.  A step is
//
//   1. stress update on the slab rows and on the ORD halo rows each side
//      (the halo rows are recomputed redundantly: same code, same inputs,
//      so bit for bit the values their owner computes);
//   2. velocity update on the slab rows only (it reads stresses up to ORD
//      rows away, all present after step 1), sources, stability;
//   3. the NH velocity rows at each edge of the slab go to a mailbox in
//      global memory (L2), then a per-block counter is released;
//   4. before the next step each block waits for its two neighbours'
//      counters and copies their edge rows into its velocity halo.
//
// So a step costs one neighbour exchange, no grid-wide barrier and no
// launch.  Every wait is bounded (globaltimer); a block that gives up
// records the step and block in `err`, every block seeing `err` returns, and
// the host reports the failure from ts_status.  The launch is cooperative,
// so all blocks are resident together (a wait on a neighbour always has a
// running neighbour to wait on).
//
// Receivers: each block writes syy at the receiver points on its rows into
// a per-step sample table; k_persist_receivers then sums every receiver's
// points in the CSR order the regular velocity kernel uses, so traces are
// the same bits.  The arithmetic of both updates is the regular kernels'
// (ts_kernels2d.cuh, family TS_TAICHI2D: sim_taichi_elastic.py:138-309 in
// the reference's operation order; TS_WGSL2D without attenuation:
// shader_webgpu_viscoelastic.wgsl:829-1072), expression for expression.
#include <cuda_runtime.h>

#include "ts_internal.cuh"

namespace ts {
namespace {

constexpr int kPOrd = 2;                 // stencil order served (acc = 2)
constexpr int kPNH = 2 * kPOrd - 1;      // velocity halo rows per side
constexpr int kPMaxThreads = 640;        // columns per block: up to 102 registers a thread

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned *p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release_u32(unsigned *p, unsigned v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// The arithmetic of the regular kernels (ts_kernels2d.cuh): FAM 0 is
// kTaichi, FAM 1 is kWgsl (sums of weighted differences divided by the grid
// step, updates times dt, velocities divided by rho).
// CPML update of one derivative with its memory in shared memory
template <int FAM>
__device__ __forceinline__ float pcpml(float d, float &psi, const Cpml &t) {
    if (FAM == 0) {
        float np_;
        const float r = taichi_cpml(d, psi, np_, t);
        psi = np_;
        return r;
    }
    psi = fmaf(t.b, psi, t.a * d);
    return qdiv(d, t.k, t.ik) + psi;
}

// one derivative term: family 0 in the reference's order, else fma with coef
template <int FAM>
__device__ __forceinline__ float pterm(float acc, const StepParams &p, int axis, int c, float hi, float lo) {
    return FAM == 0 ? taichi_term(acc, p.coef[c], hi, lo, p.od[axis]) : fmaf(p.coef[c], hi - lo, acc);
}
// the derivative from its sum: family 1 divides by the grid step
template <int FAM>
__device__ __forceinline__ float pfin(float s, const StepParams &p, int axis) {
    return FAM == 0 ? s : dscale(s, p.od[axis], p.odl[axis]);
}

template <int FAM, int R>
__global__ void __launch_bounds__(kPMaxThreads, 1) k_persist2d(const __grid_constant__ PersistArgs a) {
    constexpr int ORD = kPOrd, NH = kPNH, NV = R + 2 * NH, NS = R + 2 * ORD;
    const StepParams &p = a.p;
    extern __shared__ float sm[];
    __shared__ int s_go;
    const int W = blockDim.x;
    float *svx = sm, *svy = svx + NV * W;                  // velocity rows [x0 - NH, x0 + R + NH)
    float *ssxx = svy + NV * W, *ssyy = ssxx + NS * W;     // stress rows [x0 - ORD, x0 + R + ORD)
    float *ssxy = ssyy + NS * W;
    // CPML memories: x strips over every column ([2][NS][W] stress, [2][R][W]
    // velocity), y strips over the strip columns only ([2][NS][syw], [2][R][syw])
    const int syw = p.strip[1].width;
    float *spnx = ssxy + NS * W, *spvx = spnx + 2 * NS * W;
    float *spny = spvx + 2 * R * W, *spvy = spny + 2 * NS * syw;
    const int y = threadIdx.x, blk = blockIdx.x, G = gridDim.x;
    const int nx = p.nx, ny = p.ny, P = p.pitch;
    const int x0 = blk * R, vlo = x0 - NH, slo = x0 - ORD;
    const bool col = y < ny;
    const int sy = col ? strip_index(p.strip[1], y) : -1;

    // y-part of the update regions (ts_kernels2d.cuh)
    const bool yn = y >= ORD && y < ny - ORD + 1;
    const bool ys = y >= ORD - 1 && y < ny - ORD;
    const bool yvy = y >= ORD - 1 && y < ny - ORD;
    const bool yvx = FAM == 0 ? (y >= ORD && y < ny - ORD + 1) : (yvy && y >= ORD);

    // ---- load the slab ----
    for (int r = 0; r < NV; ++r) {
        const int x = vlo + r;
        const bool in = col && x >= 0 && x < nx;
        svx[r * W + y] = in ? p.v[0][(int64_t)x * P + y] : 0.f;
        svy[r * W + y] = in ? p.v[1][(int64_t)x * P + y] : 0.f;
    }
    float cL[NS], cM[NS], cMs[NS], cdx[R], cdy[R];   // cdx, cdy: rho at the velocity nodes
#pragma unroll
    for (int j = 0; j < NS; ++j) {
        const int x = slo + j;
        const bool in = col && x >= 0 && x < nx;
        const int64_t i = (int64_t)x * P + y;
        ssxx[j * W + y] = in ? p.s[0][i] : 0.f;
        ssyy[j * W + y] = in ? p.s[1][i] : 0.f;
        ssxy[j * W + y] = in ? p.s[3][i] : 0.f;
        cL[j] = in ? p.lam_dt[i] : 0.f;
        cM[j] = in ? p.mu_dt[i] : 0.f;
        cMs[j] = in ? p.mus_dt[0][i] : 0.f;
        const int sx = in ? strip_index(p.strip[0], x) : -1;
        spnx[(0 * NS + j) * W + y] = sx >= 0 ? p.psi[0][(int64_t)sx * P + y] : 0.f;
        spnx[(1 * NS + j) * W + y] = sx >= 0 ? p.psi[1][(int64_t)sx * P + y] : 0.f;
        if (sy >= 0) {
            spny[(0 * NS + j) * syw + sy] = in ? p.psi[2][(int64_t)x * syw + sy] : 0.f;
            spny[(1 * NS + j) * syw + sy] = in ? p.psi[3][(int64_t)x * syw + sy] : 0.f;
        }
    }
#pragma unroll
    for (int j = 0; j < R; ++j) {
        const int x = x0 + j;
        const bool in = col && x < nx;
        const int64_t i = (int64_t)x * P + y;
        cdx[j] = in ? p.dtr[0][i] : 0.f;
        cdy[j] = in ? p.dtr[1][i] : 0.f;
        const int sx = in ? strip_index(p.strip[0], x) : -1;
        spvx[(0 * R + j) * W + y] = sx >= 0 ? p.psi[4][(int64_t)sx * P + y] : 0.f;
        spvx[(1 * R + j) * W + y] = sx >= 0 ? p.psi[5][(int64_t)sx * P + y] : 0.f;
        if (sy >= 0) {
            spvy[(0 * R + j) * syw + sy] = in ? p.psi[6][(int64_t)x * syw + sy] : 0.f;
            spvy[(1 * R + j) * syw + sy] = in ? p.psi[7][(int64_t)x * syw + sy] : 0.f;
        }
    }

    const int k0 = *p.step_base, k1 = k0 + a.n_steps;
    const int q0 = a.src_start[blk], q1 = a.src_start[blk + 1];
    const int r0 = a.pts_start[blk], r1 = a.pts_start[blk + 1];
    unsigned vmax = 0u;
    bool reported = false;
    __syncthreads();

    for (int k = k0; k < k1; ++k) {
        if (k > k0) {
            // ---- wait for the neighbours' velocity rows of step k - 1 ----
            if (y == 0) {
                int go = 1;
                const unsigned want = (unsigned)k;
                const unsigned long long t0 = global_ns();
                for (;;) {
                    const bool lo_ok = blk == 0 || ld_acquire_u32(a.flags + blk - 1) >= want;
                    const bool hi_ok = blk + 1 == G || ld_acquire_u32(a.flags + blk + 1) >= want;
                    if (lo_ok && hi_ok) break;
                    if (*(volatile int *)a.err != 0) {
                        go = 0;
                        break;
                    }
                    if (global_ns() - t0 > (unsigned long long)a.wait_ns) {
                        if (atomicCAS(a.err, 0, 1) == 0) {
                            a.err[1] = k;
                            a.err[2] = blk;
                        }
                        go = 0;
                        break;
                    }
                    __nanosleep(32);
                }
                s_go = go;
            }
            __syncthreads();
            if (!s_go) return;   // uniform: every thread of the block returns here
            const int par = (k - 1) & 1;
            if (blk > 0) {   // rows [x0 - NH, x0) from the block below (its "up" edge)
                const float *m = a.mail + ((((int64_t)(blk - 1) * 2 + 1) * 2 + par) * 2) * NH * W;
#pragma unroll
                for (int r = 0; r < NH; ++r) {
                    svx[r * W + y] = __ldcg(m + (0 * NH + r) * W + y);
                    svy[r * W + y] = __ldcg(m + (1 * NH + r) * W + y);
                }
            }
            if (blk + 1 < G) {   // rows [x0 + R, x0 + R + NH) from the block above (its "down" edge)
                const float *m = a.mail + ((((int64_t)(blk + 1) * 2 + 0) * 2 + par) * 2) * NH * W;
#pragma unroll
                for (int r = 0; r < NH; ++r) {
                    svx[(R + NH + r) * W + y] = __ldcg(m + (0 * NH + r) * W + y);
                    svy[(R + NH + r) * W + y] = __ldcg(m + (1 * NH + r) * W + y);
                }
            }
            __syncthreads();
        }

        // ---- stress: normal nodes on rows slo .. slo + NS - 2, shear nodes on slo + 1 .. slo + NS - 1 ----
        if (col) {
#pragma unroll
            for (int j = 0; j < NS; ++j) {
                const int x = slo + j;
                const int jv = x - vlo;   // this row in the velocity rows
                const int sx = (x >= 0 && x < nx) ? strip_index(p.strip[0], x) : -1;
                if (j < NS - 1 && yn && x >= ORD - 1 && x < nx - ORD) {
                    float ddx = 0.f, ddy = 0.f;
#pragma unroll
                    for (int c = 0; c < ORD; ++c) {
                        ddx = pterm<FAM>(ddx, p, 0, c, svx[(jv + c + 1) * W + y], svx[(jv - c) * W + y]);
                        ddy = pterm<FAM>(ddy, p, 1, c, svy[jv * W + y + c], svy[jv * W + y - c - 1]);
                    }
                    ddx = pfin<FAM>(ddx, p, 0);
                    ddy = pfin<FAM>(ddy, p, 1);
                    if (sx >= 0) ddx = pcpml<FAM>(ddx, spnx[(0 * NS + j) * W + y], p.tab_h[0][x]);
                    if (sy >= 0) ddy = pcpml<FAM>(ddy, spny[(0 * NS + j) * syw + sy], p.tab_f[1][y]);
                    const float L = cL[j], M = cM[j];
                    float sxx = ssxx[j * W + y], syy = ssyy[j * W + y];
                    if (FAM == 0) {
                        const float dl = __fmul_rn(L, __fadd_rn(ddx, ddy));
                        sxx = taichi_normal(sxx, dl, M, ddx, p.dt);
                        syy = taichi_normal(syy, dl, M, ddy, p.dt);
                    } else {
                        const float L2M = fmaf(2.f, M, L);
                        const float ux = fmaf(L2M, ddx, L * ddy), uy = fmaf(L, ddx, L2M * ddy);
                        sxx += ux * p.dt;
                        syy += uy * p.dt;
                    }
                    ssxx[j * W + y] = sxx;
                    ssyy[j * W + y] = syy;
                }
                if (j > 0 && ys && x >= ORD && x < nx - ORD + 1) {
                    float av = 0.f, bv = 0.f;
#pragma unroll
                    for (int c = 0; c < ORD; ++c) {
                        av = pterm<FAM>(av, p, 0, c, svy[(jv + c) * W + y], svy[(jv - c - 1) * W + y]);
                        bv = pterm<FAM>(bv, p, 1, c, svx[jv * W + y + c + 1], svx[jv * W + y - c]);
                    }
                    av = pfin<FAM>(av, p, 0);
                    bv = pfin<FAM>(bv, p, 1);
                    if (sx >= 0) av = pcpml<FAM>(av, spnx[(1 * NS + j) * W + y], p.tab_f[0][x]);
                    if (sy >= 0) bv = pcpml<FAM>(bv, spny[(1 * NS + j) * syw + sy], p.tab_h[1][y]);
                    if (FAM == 0) {
                        ssxy[j * W + y] = taichi_shear(ssxy[j * W + y], __fadd_rn(av, bv), cMs[j], p.dt);
                    } else {
                        const float e = av + bv;
                        const float u = cMs[j] * e;
                        ssxy[j * W + y] = ssxy[j * W + y] + u * p.dt;
                    }
                }
            }
        }
        __syncthreads();

        // ---- receiver samples of syy on this block's rows ----
        for (int q = r0 + y; q < r1; q += W) {
            const int4 pt = a.pts[q];   // (row in the slab, column, CSR position, -)
            a.samples[(int64_t)k * a.n_pts + pt.z] = ssyy[(pt.x + ORD) * W + pt.y];
        }

        // ---- velocity on the slab rows, sources, stability, edge rows to the mailbox ----
        if (col) {
            float *mdn = a.mail + ((((int64_t)blk * 2 + 0) * 2 + (k & 1)) * 2) * NH * W;
            float *mup = a.mail + ((((int64_t)blk * 2 + 1) * 2 + (k & 1)) * 2) * NH * W;
#pragma unroll
            for (int j = 0; j < R; ++j) {
                const int x = x0 + j;
                if (x >= nx) break;
                const int js = x - slo, jv = x - vlo;
                const int sx = strip_index(p.strip[0], x);
                const bool in_vy = yvy && x >= ORD - 1 && x < nx - ORD;
                const bool in_vx = FAM == 0 ? (yvx && x >= ORD && x < nx - ORD + 1) : (yvx && in_vy && x >= ORD);
                float vxn = 0.f, vyn = 0.f;
                if (in_vx) {
                    float av = 0.f, bv = 0.f;
#pragma unroll
                    for (int c = 0; c < ORD; ++c) {
                        av = pterm<FAM>(av, p, 0, c, ssxx[(js + c) * W + y], ssxx[(js - c - 1) * W + y]);
                        bv = pterm<FAM>(bv, p, 1, c, ssxy[js * W + y + c], ssxy[js * W + y - c - 1]);
                    }
                    av = pfin<FAM>(av, p, 0);
                    bv = pfin<FAM>(bv, p, 1);
                    if (sx >= 0) av = pcpml<FAM>(av, spvx[(0 * R + j) * W + y], p.tab_f[0][x]);
                    if (sy >= 0) bv = pcpml<FAM>(bv, spvy[(0 * R + j) * syw + sy], p.tab_f[1][y]);
                    if (FAM == 0) {
                        vxn = taichi_velocity(svx[jv * W + y], __fadd_rn(av, bv), 0.f, cdx[j], p.dt);
                    } else {
                        vxn = wgsl_velocity_rho(svx[jv * W + y], av + bv, cdx[j], p.dt);
                    }
                }
                if (in_vy) {
                    float av = 0.f, bv = 0.f;
#pragma unroll
                    for (int c = 0; c < ORD; ++c) {
                        av = pterm<FAM>(av, p, 0, c, ssxy[(js + c + 1) * W + y], ssxy[(js - c) * W + y]);
                        bv = pterm<FAM>(bv, p, 1, c, ssyy[js * W + y + c + 1], ssyy[js * W + y - c]);
                    }
                    av = pfin<FAM>(av, p, 0);
                    bv = pfin<FAM>(bv, p, 1);
                    if (sx >= 0) av = pcpml<FAM>(av, spvx[(1 * R + j) * W + y], p.tab_h[0][x]);
                    if (sy >= 0) bv = pcpml<FAM>(bv, spvy[(1 * R + j) * syw + sy], p.tab_h[1][y]);
                    if (FAM == 0) {
                        float src = 0.f;   // the source joins the update inside it (as the regular kernel)
                        for (int q = q0; q < q1; ++q) {
                            const int4 s = a.srcs[q];   // (row in the slab, column, table column, rho bits)
                            if (s.x == j && s.y == y && k < p.src_rows)
                                src = __fdiv_rn(__fmul_rn(__ldg(p.src_tab + (int64_t)k * p.src_ncol + s.z), p.dt),
                                                __int_as_float(s.w));
                        }
                        vyn = taichi_velocity(svy[jv * W + y], __fadd_rn(av, bv), src, cdy[j], p.dt);
                    } else {
                        vyn = wgsl_velocity_rho(svy[jv * W + y], av + bv, cdy[j], p.dt);
                    }
                }
                if (FAM != 0) {
                    for (int q = q0; q < q1; ++q) {
                        const int4 s = a.srcs[q];   // (row in the slab, column, table column, rho bits)
                        if (s.x == j && s.y == y && k < p.src_rows)
                            vyn += wgsl_source(__ldg(p.src_tab + (int64_t)k * p.src_ncol + s.z), __int_as_float(s.w), p.dt);
                    }
                }
                svx[jv * W + y] = vxn;
                svy[jv * W + y] = vyn;
                if (j < NH) {
                    __stcg(mdn + (0 * NH + j) * W + y, vxn);
                    __stcg(mdn + (1 * NH + j) * W + y, vyn);
                }
                if (j >= R - NH) {
                    __stcg(mup + (0 * NH + j - (R - NH)) * W + y, vxn);
                    __stcg(mup + (1 * NH + j - (R - NH)) * W + y, vyn);
                }
                const float v2 = fmaf(vxn, vxn, vyn * vyn);
                if (!(v2 <= p.v2_threshold) && !reported) {
                    atomicMin(p.first_bad, k);
                    reported = true;
                }
                vmax = max(vmax, __float_as_uint(v2));
            }
        }
        __syncthreads();
        if (y == 0) {
            __threadfence();
            if (blk != a.stall_block) st_release_u32(a.flags + blk, (unsigned)(k + 1));
        }
    }

    // ---- write the slab back, once both neighbours are past their last step
    // (they read rows of this slab from global memory when they started) ----
    if (y == 0) {
        int go = 1;
        const unsigned long long t0 = global_ns();
        for (;;) {
            const bool lo_ok = blk == 0 || ld_acquire_u32(a.flags + blk - 1) >= (unsigned)k1;
            const bool hi_ok = blk + 1 == G || ld_acquire_u32(a.flags + blk + 1) >= (unsigned)k1;
            if (lo_ok && hi_ok) break;
            if (*(volatile int *)a.err != 0) {
                go = 0;
                break;
            }
            if (global_ns() - t0 > (unsigned long long)a.wait_ns) {
                if (atomicCAS(a.err, 0, 1) == 0) {
                    a.err[1] = k1;
                    a.err[2] = blk;
                }
                go = 0;
                break;
            }
            __nanosleep(32);
        }
        s_go = go;
    }
    __syncthreads();
    if (!s_go) return;
    if (col) {
#pragma unroll
        for (int j = 0; j < R; ++j) {
            const int x = x0 + j;
            if (x >= nx) break;
            const int64_t i = (int64_t)x * P + y;
            const int js = x - slo, jv = x - vlo;
            p.v[0][i] = svx[jv * W + y];
            p.v[1][i] = svy[jv * W + y];
            p.s[0][i] = ssxx[js * W + y];
            p.s[1][i] = ssyy[js * W + y];
            p.s[3][i] = ssxy[js * W + y];
            const int sx = strip_index(p.strip[0], x);
            if (sx >= 0) {
                const int64_t ix = (int64_t)sx * P + y;
                p.psi[0][ix] = spnx[(0 * NS + js) * W + y];
                p.psi[1][ix] = spnx[(1 * NS + js) * W + y];
                p.psi[4][ix] = spvx[(0 * R + j) * W + y];
                p.psi[5][ix] = spvx[(1 * R + j) * W + y];
            }
            if (sy >= 0) {
                const int64_t iy = (int64_t)x * syw + sy;
                p.psi[2][iy] = spny[(0 * NS + js) * syw + sy];
                p.psi[3][iy] = spny[(1 * NS + js) * syw + sy];
                p.psi[6][iy] = spvy[(0 * R + j) * syw + sy];
                p.psi[7][iy] = spvy[(1 * R + j) * syw + sy];
            }
        }
    }
    const unsigned m = __reduce_max_sync(0xffffffffu, vmax);
    if ((y & 31) == 0) atomicMax(reinterpret_cast<unsigned *>(p.block_max) + blk % a.n_blocks, m);
}

// traces[k][g] = sum of the samples of receiver g's points, in CSR order,
// for k in [*step_base, *step_base + n) with k >= first[g] (the regular
// velocity kernel's sum, same order).
__global__ void k_persist_receivers(const StepParams p, const float *samples, int n_pts, int n) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= p.n_rec) return;
    const int first = __ldg(p.rec_first_step + g), q0 = __ldg(p.rec_start + g), q1 = __ldg(p.rec_start + g + 1);
    for (int j = blockIdx.y; j < n; j += gridDim.y) {
        const int k = *p.step_base + j;
        if (k < first) continue;
        float acc = 0.f;
        for (int q = q0; q < q1; ++q) acc += samples[(int64_t)k * n_pts + q];
        p.traces[(int64_t)k * p.n_rec + g] = acc;
    }
}

template <int FAM, int R>
cudaError_t launch_fr(const PersistArgs &a, int grid, int threads, size_t smem, cudaStream_t st) {
    cudaError_t e = cudaFuncSetAttribute(k_persist2d<FAM, R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(threads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k_persist2d<FAM, R>, a);
}

template <int FAM, int R>
int max_blocks(int threads, size_t smem) {
    if (cudaFuncSetAttribute(k_persist2d<FAM, R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return 0;
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_persist2d<FAM, R>, threads, smem) != cudaSuccess) return 0;
    return nb;
}

}  // namespace

size_t persist_2d_smem(int rows, int threads, int strip_y) {
    const int NV = rows + 2 * kPNH, NS = rows + 2 * kPOrd;
    return ((size_t)(2 * NV + 3 * NS + 2 * NS + 2 * rows) * threads + (size_t)(2 * NS + 2 * rows) * strip_y) *
           sizeof(float);
}

int persist_2d_plan(int family, int ord, int zen_mode, int nx, int ny, int strip_y, int n_sms, int *rows,
                    int *blocks, int *threads, size_t *smem) {
    if (ord != kPOrd || zen_mode != 0 || (family != 0 && family != 1)) return 0;
    const int t = (ny + 31) / 32 * 32;
    if (t > kPMaxThreads || nx < 2 * kPNH) return 0;
    for (int r : {4, 5}) {
        const int g = (nx + r - 1) / r;
        const size_t s = persist_2d_smem(r, t, strip_y);
        if (s > 227 * 1024) continue;
        const int nb = family == 0 ? (r == 4 ? max_blocks<0, 4>(t, s) : max_blocks<0, 5>(t, s))
                                   : (r == 4 ? max_blocks<1, 4>(t, s) : max_blocks<1, 5>(t, s));
        if (nb < 1 || g > nb * n_sms) continue;
        *rows = r;
        *blocks = g;
        *threads = t;
        *smem = s;
        return 1;
    }
    return 0;
}

cudaError_t launch_persist_2d_receivers(const PersistArgs &a, int n_steps, cudaStream_t st) {
    if (a.p.n_rec <= 0 || n_steps <= 0) return cudaSuccess;
    const dim3 grid((a.p.n_rec + 127) / 128, n_steps < 4096 ? n_steps : 4096);
    k_persist_receivers<<<grid, 128, 0, st>>>(a.p, a.samples, a.n_pts, n_steps);
    return cudaGetLastError();
}

cudaError_t launch_persist_2d(const PersistArgs &a, int family, int rows, int blocks, int threads, size_t smem,
                              cudaStream_t st) {
    if (a.n_steps <= 0) return cudaSuccess;
    cudaError_t e;
    if (family == 0) e = rows == 4 ? launch_fr<0, 4>(a, blocks, threads, smem, st) : launch_fr<0, 5>(a, blocks, threads, smem, st);
    else e = rows == 4 ? launch_fr<1, 4>(a, blocks, threads, smem, st) : launch_fr<1, 5>(a, blocks, threads, smem, st);
    if (e != cudaSuccess) return e;
    return launch_persist_2d_receivers(a, a.n_steps, st);
}

}  // namespace ts
