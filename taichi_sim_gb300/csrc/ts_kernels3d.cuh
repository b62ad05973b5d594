// 3D staggered-grid (visco)elastic step kernels on sm_103a (internal header,
// included by the translation units that instantiate them).
//
// One time step = three launches: k_normal3d (sxx, syy, szz), k_shear3d
// (sxy, sxz, syz), each with its CPML strips and Zener update fused, then
// k_velocity3d (vx, vy, vz with CPML, Dirichlet zeroing, source injection,
// receiver sampling of szz and stability bookkeeping fused).  Splitting the
// stress update halves the live state of a thread, so more blocks stay
// resident per SM.  A thread owns one (y, z) column (z is the contiguous
// axis; the 8 warps of a block cover kZW3 32-node runs along z by 8 / kZW3
// rows along y) and updates consecutive nodes along x; the x-derivatives
// come from register windows that take one new plane per node, the y- and
// z-derivatives from loads.
// As in 2D, every load of a node is issued before its first store so that
// one memory latency is paid per node.
//
// Semantics: family TS_WGSL3D, shader_webgpu_3D_viscoelastic.wgsl:1341-1773
// and :1824-1843, including its quirks (normal stresses use point
// rho/cp/cs, shear moduli average rho and cs over 4 nodes without the
// cs == 0 test, vz uses the vy-node density, all three velocities are zeroed
// outside the vz region, the source drives vz).
//
// Arithmetic: as the shaders, every derivative divided by its grid step,
// every update multiplied by dt and every velocity update divided by rho;
// the constants 1 / d and dt / rho enter as pairs (hi, lo) exact to ~48 bits,
// so that no rounded constant (coef / d, lambda dt, dt / rho) biases every
// node and step alike; sums contract to fma.
//
// Coefficients: with PAL the stress kernels take the per-node coefficients
// from a palette (one 16-bit index per node into a table of the model's
// distinct coefficient tuples, ts_internal.cuh: Pal3), otherwise from one
// array per coefficient; the velocity kernel reads its dt / rho pairs from
// arrays (a variant reading them from a palette table measured slower).
#pragma once
#include <cuda_runtime.h>

#include <type_traits>
#include "ts_internal.cuh"

namespace ts {
namespace {

// b * psi + a * d, then d / k + psi (the division as the shader's)
__device__ __forceinline__ float cpml(float d, float psi_old, float &psi_new, const Cpml &t) {
    psi_new = fmaf(t.b, psi_old, t.a * d);
    return qdiv(d, t.k, t.ik) + psi_new;
}

// Load of a field value written by an earlier kernel of the stream.  With
// programmatic dependent launch that kernel's lifetime overlaps this one's,
// so the field is not read-only for this kernel's lifetime and must not be
// read through the non-coherent path (measured: stale values, wrong results
// in a few percent of runs); ld.global.ca is coherent after
// griddepcontrol.wait and still cached in L1.
__device__ __forceinline__ float fld(const float *q) { return __ldca(q); }

// Stencil values of one staggered derivative: hi[c] - lo[c] pairs.
// PLUS: f[i + (c+1) s] - f[i - c s]; otherwise f[i + c s] - f[i - (c+1) s].
template <int ORD>
struct Pairs {
    float hi[ORD], lo[ORD];
};

template <int ORD, bool PLUS, typename I>
__device__ __forceinline__ Pairs<ORD> load_pairs(const float *f, I i, I s) {
    Pairs<ORD> r;
#pragma unroll
    for (int c = 0; c < ORD; ++c) {
        r.hi[c] = fld(f + i + (PLUS ? (c + 1) : c) * s);
        r.lo[c] = fld(f + i - (PLUS ? c : (c + 1)) * s);
    }
    return r;
}

// sum_c coef[c] (hi[c] - lo[c]) / d_axis: the shader divides every term by
// the grid step (wgsl3d:1367-1369); the sum is divided once, so that no
// rounding of coef / d biases every derivative alike
template <int ORD>
__device__ __forceinline__ float deriv(const Pairs<ORD> &q, const StepParams &p, int axis) {
    float a = 0.f;
#pragma unroll
    for (int c = 0; c < ORD; ++c) a = fmaf(p.coef[c], q.hi[c] - q.lo[c], a);
    return dscale(a, p.od[axis], p.odl[axis]);
}

// Resident blocks per SM the kernels are compiled for (register budgets 64
// and 85 per thread; measured against 1 to 4 on the 256^3 case).
#ifndef TS_VELOCITY3D_MIN_BLOCKS
#define TS_VELOCITY3D_MIN_BLOCKS 3
#endif
#ifndef TS_STRESS3D_MIN_BLOCKS
#define TS_STRESS3D_MIN_BLOCKS 4
#endif
constexpr int kStressMinBlocks = TS_STRESS3D_MIN_BLOCKS, kVelocityMinBlocks = TS_VELOCITY3D_MIN_BLOCKS;
// x window of 2*ORD planes of one field at (y, z), first plane r0; planes
// outside the grid read 0
// (CHECK = false: every plane is known to lie inside the grid)
template <int ORD, bool CHECK = true, typename I>
__device__ __forceinline__ void xwindow(float (&w)[2 * ORD], const float *f, int r0, int nx, I X, I yz) {
#pragma unroll
    for (int j = 0; j < 2 * ORD; ++j) {
        const int r = r0 + j;
        w[j] = (!CHECK || (r >= 0 && r < nx)) ? fld(f + r * X + yz) : 0.f;
    }
}

template <int ORD, bool CHECK = true, typename I>
__device__ __forceinline__ void xshift(float (&w)[2 * ORD], const float *f, int r_new, int nx, I X, I yz) {
#pragma unroll
    for (int j = 0; j < 2 * ORD - 1; ++j) w[j] = w[j + 1];
    w[2 * ORD - 1] = (!CHECK || (r_new >= 0 && r_new < nx)) ? fld(f + r_new * X + yz) : 0.f;
}

// A warp whose TX-node chunks lie wholly in the interior (every node inside
// the update regions of all three kernels, outside the CPML strips, window
// planes inside the grid) sweeps without per-node region, strip or bounds
// tests.  Evaluated by all 32 lanes before any of them returns.
template <int ORD, int TX>
__device__ __forceinline__ bool interior_warp(const StepParams &p, int y, int z, int x0, int sy, int sz) {
    const bool lane = y < p.ny && z < p.nz && sy < 0 && sz < 0 && y >= ORD && y < p.ny - ORD && z >= ORD &&
                      z < p.nz - ORD && x0 >= ORD && x0 >= p.strip[0].lo && x0 + TX + ORD <= p.nx &&
                      x0 + TX <= p.strip[0].hi;
    return __all_sync(0xffffffffu, lane);
}

// A warp interior along x and y (its TX-node chunk and its y row outside
// the x and y strips and away from those grid edges) whose z run may cross
// a z strip or the z edge: its per-node x and y tests compile out, the z
// tests are per lane.
template <int ORD, int TX>
__device__ __forceinline__ bool xy_interior_warp(const StepParams &p, int y, int z, int x0, int sy) {
    const bool lane = y < p.ny && sy < 0 && y >= ORD && y < p.ny - ORD && x0 >= ORD && x0 >= p.strip[0].lo &&
                      x0 + TX + ORD <= p.nx && x0 + TX <= p.strip[0].hi;
    return __all_sync(0xffffffffu, lane);
}

// sum_c coef[c] (w[ORD + c] - w[ORD - 1 - c]) / dx
template <int ORD>
__device__ __forceinline__ float wderiv(const float (&w)[2 * ORD], const StepParams &p) {
    float a = 0.f;
#pragma unroll
    for (int c = 0; c < ORD; ++c) a = fmaf(p.coef[c], w[ORD + c] - w[ORD - 1 - c], a);
    return dscale(a, p.od[0], p.odl[0]);
}

// Normal stresses (sxx, syy, szz, their Zener memory variables and CPML
// strips), x-marching: thread (z, y) updates kTX3S consecutive nodes along x,
// the x-derivative of vx from a register window, the y- and z-derivatives
// from loads.
template <int ORD, int ZM, int NS, typename I, bool PAL>
__device__ __forceinline__ void normal3d_body(const StepParams &p, int bz) {
    const int z = blockIdx.x * kZB3 + (threadIdx.y % kZW3) * kBX3 + threadIdx.x;
    const int y = blockIdx.y * kYB3 + threadIdx.y / kZW3;
    const int x0 = bz * kTX3S;
    if (y >= p.ny || z >= p.nz || x0 >= p.nx) return;
    const I X = (I)p.plane, Y = (I)p.pitch, yz = (I)y * Y + z, G = (I)p.grid_elems;
    const float *__restrict__ vx = p.v[0];
    const float *__restrict__ vy = p.v[1];
    const float *__restrict__ vz = p.v[2];
    const bool yz_n = y >= ORD && y < p.ny - ORD + 1 && z >= ORD && z < p.nz - ORD + 1;
    const int sy = strip_index(p.strip[1], y), sz = strip_index(p.strip[2], z);
    const int n_mech = NS == 3 ? 3 : p.zen.n;
    constexpr int R = NS > 0 ? NS : 1;
    // L2 prefetch of the nodes' stresses and memory variables (last written
    // two launches back): mode 1 the later nodes after the wait, mode 2 every
    // node before it, overlapping the previous launch's drain
    if (p.prefetch_3d == 2 && yz_n) {
#pragma unroll
        for (int t = 0; t < kTX3S; ++t) {
            const int x = x0 + t;
            if (x >= ORD - 1 && x < p.nx - ORD) {
                const I i = (I)x * X + yz;
                prefetch_l2(p.s[0] + i);
                prefetch_l2(p.s[1] + i);
                prefetch_l2(p.s[2] + i);
                if (ZM != 0)
                    for (int l = 0; l < n_mech; ++l) {
                        prefetch_l2(p.r[0] + l * G + i);
                        prefetch_l2(p.r[1] + l * G + i);
                        prefetch_l2(p.r[2] + l * G + i);
                    }
            }
        }
    }
    pdl_wait();
    if (p.prefetch_3d == 1 && yz_n) {   // the later nodes' stresses and memory variables
#pragma unroll
        for (int t = 1; t < kTX3S; ++t) {
            const int x = x0 + t;
            if (x >= ORD - 1 && x < p.nx - ORD) {
                const I i = (I)x * X + yz;
                prefetch_l2(p.s[0] + i);
                prefetch_l2(p.s[1] + i);
                prefetch_l2(p.s[2] + i);
                if (ZM != 0)
                    for (int l = 0; l < n_mech; ++l) {
                        prefetch_l2(p.r[0] + l * G + i);
                        prefetch_l2(p.r[1] + l * G + i);
                        prefetch_l2(p.r[2] + l * G + i);
                    }
            }
        }
    }
    float wx[2 * ORD];   // vx planes [x-ORD+1, x+ORD]
    xwindow<ORD>(wx, vx, x0 - ORD + 1, p.nx, X, yz);
#pragma unroll
    for (int t = 0; t < kTX3S; ++t) {
        const int x = x0 + t;
        if (x >= p.nx) break;
        if (yz_n && x >= ORD - 1 && x < p.nx - ORD) {
            const I i = (I)x * X + yz;
            const int sx = strip_index(p.strip[0], x);
            const I ix = ((I)sx * p.ny + y) * Y + z;
            const I iy = ((I)x * p.strip[1].width + sy) * Y + z;
            const I iz = ((I)x * p.ny + y) * p.strip[2].width + sz;
            // ---- loads ----
            const Pairs<ORD> n_y = load_pairs<ORD, false>(vy, i, Y);   // vy[y+c]-vy[y-c-1]
            const Pairs<ORD> n_z = load_pairs<ORD, false>(vz, i, (I)1);   // vz[z+c]-vz[z-c-1]
            // palette: the index first, its table entry after every other load
            // (the entry load waits for the index)
            const uint16_t pidx = PAL ? __ldg(p.pal_idx + i) : 0;
            float L = 0.f, M = 0.f, gp = 1.f, gs = 1.f;
            if constexpr (!PAL) {
                L = __ldg(p.lam_dt + i);
                M = __ldg(p.mu_dt + i);
                if (ZM == 2) {
                    gp = __ldg(p.g_p + i);
                    gs = __ldg(p.g_s + i);
                }
            }
            const float s0 = p.s[0][i], s1 = p.s[1][i], s2 = p.s[2][i];
            float pz0 = 0.f, pz1 = 0.f, pz2 = 0.f;
            if (sx >= 0) pz0 = p.psi[0][ix];
            if (sy >= 0) pz1 = p.psi[1][iy];
            if (sz >= 0) pz2 = p.psi[2][iz];
            float r0[R], r1[R], r2[R];
            if (ZM != 0) {
#pragma unroll
                for (int l = 0; l < R; ++l)
                    if (l < n_mech) {
                        r0[l] = p.r[0][l * G + i];
                        r1[l] = p.r[1][l * G + i];
                        r2[l] = p.r[2][l * G + i];
                    }
            }
            if constexpr (PAL) {
                const float4 c = __ldg(&p.pal[pidx].normal);
                L = c.x;
                M = c.y;
                if (ZM == 2) {
                    gp = c.z;
                    gs = c.w;
                }
            }
            // ---- update: vx[x+c+1]-vx[x-c] from the window ----
            float ddx = wderiv<ORD>(wx, p), ddy = deriv(n_y, p, 1), ddz = deriv(n_z, p, 2);
            float np_;
            if (sx >= 0) {
                ddx = cpml(ddx, pz0, np_, p.tab_h[0][x]);
                p.psi[0][ix] = np_;
            }
            if (sy >= 0) {
                ddy = cpml(ddy, pz1, np_, p.tab_f[1][y]);
                p.psi[1][iy] = np_;
            }
            if (sz >= 0) {
                ddz = cpml(ddz, pz2, np_, p.tab_f[2][z]);
                p.psi[2][iz] = np_;
            }
            const float L2M = fmaf(2.f, M, L);
            float ux = fmaf(L2M, ddx, L * (ddy + ddz));
            float uy = fmaf(L2M, ddy, L * (ddx + ddz));
            float uz = fmaf(L2M, ddz, L * (ddx + ddy));
            if (ZM != 0) {
                const float div = ddx + ddy + ddz;
                const float third = div * (1.f / 3.f);
                const float dy_ = ddx - third, dz_ = ddy - third;
                float srxx = 0.f, sryy = 0.f, srzz = 0.f;
#pragma unroll
                for (int l = 0; l < R; ++l)
                    if (l < n_mech) {
                        const float a = fmaf(p.zen.Ap[l], r0[l], (p.zen.Bp[l] * gp) * div);
                        const float b = fmaf(p.zen.As[l], r1[l], (p.zen.Bs[l] * gs) * dy_);
                        const float c = fmaf(p.zen.As[l], r2[l], (p.zen.Bs[l] * gs) * dz_);
                        srxx += r0[l] + a;
                        sryy += r1[l] + b;
                        srzz += r2[l] + c;
                        p.r[0][l * G + i] = a;
                        p.r[1][l * G + i] = b;
                        p.r[2][l * G + i] = c;
                    }
                const float hl23 = 0.5f * fmaf(2.f / 3.f, M, L);
                ux = fmaf(hl23, srxx, fmaf(M, sryy, ux));
                uy = fmaf(hl23, srxx, fmaf(M, srzz, uy));
                uz = fmaf(0.5f * L2M, srxx, fmaf(-M * (1.f / 3.f), sryy + srzz, uz));
            }
            p.s[0][i] = s0 + ux * p.dt;   // (...) dt, wgsl3d:1442-1449
            p.s[1][i] = s1 + uy * p.dt;
            p.s[2][i] = s2 + uz * p.dt;
        }
        if (t + 1 < kTX3S) xshift<ORD>(wx, vx, x + ORD + 1, p.nx, X, yz);
    }
    pdl_trigger();
}

// Shear stresses (sxy, sxz, syz with their Zener memory variables and CPML
// strips), x-marching as k_normal3d: the x-derivatives of vy and vz from
// register windows.
template <int ORD, int ZM, int NS, typename I, bool PAL>
__device__ __forceinline__ void shear3d_body(const StepParams &p, int bz) {
    const int z = blockIdx.x * kZB3 + (threadIdx.y % kZW3) * kBX3 + threadIdx.x;
    const int y = blockIdx.y * kYB3 + threadIdx.y / kZW3;
    const int x0 = bz * kTX3S;
    if (y >= p.ny || z >= p.nz || x0 >= p.nx) return;
    const I X = (I)p.plane, Y = (I)p.pitch, yz = (I)y * Y + z, G = (I)p.grid_elems;
    const float *__restrict__ vx = p.v[0];
    const float *__restrict__ vy = p.v[1];
    const float *__restrict__ vz = p.v[2];
    const bool yz_s = y >= ORD - 1 && y < p.ny - ORD && z >= ORD - 1 && z < p.nz - ORD;
    const int sy = strip_index(p.strip[1], y), sz = strip_index(p.strip[2], z);
    const int n_mech = NS == 3 ? 3 : p.zen.n;
    constexpr int R = NS > 0 ? NS : 1;
    if (p.prefetch_3d == 2 && yz_s) {   // as in normal3d_body
#pragma unroll
        for (int t = 0; t < kTX3S; ++t) {
            const int x = x0 + t;
            if (x >= ORD - 1 && x < p.nx - ORD + 1) {
                const I i = (I)x * X + yz;
                prefetch_l2(p.s[3] + i);
                prefetch_l2(p.s[4] + i);
                prefetch_l2(p.s[5] + i);
                if (ZM != 0)
                    for (int l = 0; l < n_mech; ++l) {
                        prefetch_l2(p.r[3] + l * G + i);
                        prefetch_l2(p.r[4] + l * G + i);
                        prefetch_l2(p.r[5] + l * G + i);
                    }
            }
        }
    }
    pdl_wait();
    if (p.prefetch_3d == 1 && yz_s) {   // the later nodes' stresses and memory variables
#pragma unroll
        for (int t = 1; t < kTX3S; ++t) {
            const int x = x0 + t;
            if (x >= ORD - 1 && x < p.nx - ORD + 1) {
                const I i = (I)x * X + yz;
                prefetch_l2(p.s[3] + i);
                prefetch_l2(p.s[4] + i);
                prefetch_l2(p.s[5] + i);
                if (ZM != 0)
                    for (int l = 0; l < n_mech; ++l) {
                        prefetch_l2(p.r[3] + l * G + i);
                        prefetch_l2(p.r[4] + l * G + i);
                        prefetch_l2(p.r[5] + l * G + i);
                    }
            }
        }
    }
    float wy[2 * ORD], wz[2 * ORD];   // vy and vz planes [x-ORD, x+ORD-1]
    xwindow<ORD>(wy, vy, x0 - ORD, p.nx, X, yz);
    xwindow<ORD>(wz, vz, x0 - ORD, p.nx, X, yz);
#pragma unroll
    for (int t = 0; t < kTX3S; ++t) {
        const int x = x0 + t;
        if (x >= p.nx) break;
        const bool in_xy = yz_s && x >= ORD && x < p.nx - ORD + 1;
        const bool in_yz = yz_s && x >= ORD - 1 && x < p.nx - ORD;
        if (in_xy || in_yz) {
            const I i = (I)x * X + yz;
            const int sx = strip_index(p.strip[0], x);
            const I ix = ((I)sx * p.ny + y) * Y + z;
            const I iy = ((I)x * p.strip[1].width + sy) * Y + z;
            const I iz = ((I)x * p.ny + y) * p.strip[2].width + sz;
            // ---- loads ----
            Pairs<ORD> a_vx, b_vx, c_vz, c_vy;
            float Mxy = 0.f, Mxz = 0.f, Myz = 0.f, s_xy = 0.f, s_xz = 0.f, s_yz = 0.f;
            float psi[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
            float r3[R], r4[R], r5[R];
            // palette: the index first, its table entry after every other load
            const uint16_t pidx = PAL ? __ldg(p.pal_idx + i) : 0;
            float gs = 1.f;
            if (!PAL && ZM == 2) gs = __ldg(p.g_s + i);
            if (in_xy) {
                a_vx = load_pairs<ORD, true>(vx, i, Y);   // vx[y+c+1]-vx[y-c]
                b_vx = load_pairs<ORD, true>(vx, i, (I)1);   // vx[z+c+1]-vx[z-c]
                if (!PAL) {
                    Mxy = __ldg(p.mus_dt[0] + i);
                    Mxz = __ldg(p.mus_dt[1] + i);
                }
                s_xy = p.s[3][i];
                s_xz = p.s[4][i];
                if (sx >= 0) {
                    psi[0] = p.psi[3][ix];
                    psi[2] = p.psi[5][ix];
                }
                if (sy >= 0) psi[1] = p.psi[4][iy];
                if (sz >= 0) psi[3] = p.psi[6][iz];
                if (ZM != 0) {
#pragma unroll
                    for (int l = 0; l < R; ++l)
                        if (l < n_mech) {
                            r3[l] = p.r[3][l * G + i];
                            r4[l] = p.r[4][l * G + i];
                        }
                }
            }
            if (in_yz) {
                c_vz = load_pairs<ORD, true>(vz, i, Y);   // vz[y+c+1]-vz[y-c]
                c_vy = load_pairs<ORD, true>(vy, i, (I)1);   // vy[z+c+1]-vy[z-c]
                if (!PAL) Myz = __ldg(p.mus_dt[2] + i);
                s_yz = p.s[5][i];
                if (sy >= 0) psi[4] = p.psi[7][iy];
                if (sz >= 0) psi[5] = p.psi[8][iz];
                if (ZM != 0) {
#pragma unroll
                    for (int l = 0; l < R; ++l)
                        if (l < n_mech) r5[l] = p.r[5][l * G + i];
                }
            }
            if constexpr (PAL) {
                const float4 c = __ldg(&p.pal[pidx].shear);
                Mxy = c.x;
                Mxz = c.y;
                Myz = c.z;
                if (ZM == 2) gs = c.w;
            }
            float np_;
            // ---- sigma_xy: vy[x+c]-vy[x-c-1] (window), sigma_xz: vz[x+c]-vz[x-c-1] (window) ----
            if (in_xy) {
                float a1 = wderiv<ORD>(wy, p), a2 = deriv(a_vx, p, 1);
                float b1 = wderiv<ORD>(wz, p), b2 = deriv(b_vx, p, 2);
                if (sx >= 0) {
                    a1 = cpml(a1, psi[0], np_, p.tab_f[0][x]);
                    p.psi[3][ix] = np_;
                    b1 = cpml(b1, psi[2], np_, p.tab_f[0][x]);
                    p.psi[5][ix] = np_;
                }
                if (sy >= 0) {
                    a2 = cpml(a2, psi[1], np_, p.tab_h[1][y]);
                    p.psi[4][iy] = np_;
                }
                if (sz >= 0) {
                    b2 = cpml(b2, psi[3], np_, p.tab_h[2][z]);
                    p.psi[6][iz] = np_;
                }
                const float ea = a1 + a2, eb = b1 + b2;
                float u = Mxy * ea, w = Mxz * eb;
                if (ZM != 0) {
                    float sa = 0.f, sb = 0.f;
#pragma unroll
                    for (int l = 0; l < R; ++l)
                        if (l < n_mech) {
                            const float na = fmaf(p.zen.As[l], r3[l], (p.zen.Bs[l] * gs) * ea);
                            const float nb = fmaf(p.zen.As[l], r4[l], (p.zen.Bs[l] * gs) * eb);
                            sa += r3[l] + na;
                            sb += r4[l] + nb;
                            p.r[3][l * G + i] = na;
                            p.r[4][l * G + i] = nb;
                        }
                    u = fmaf(0.5f * Mxy, sa, u);
                    w = fmaf(0.5f * Mxz, sb, w);
                }
                p.s[3][i] = s_xy + u * p.dt;
                p.s[4][i] = s_xz + w * p.dt;
            }
            // ---- sigma_yz ----
            if (in_yz) {
                float a1 = deriv(c_vz, p, 1), a2 = deriv(c_vy, p, 2);
                if (sy >= 0) {
                    a1 = cpml(a1, psi[4], np_, p.tab_h[1][y]);
                    p.psi[7][iy] = np_;
                }
                if (sz >= 0) {
                    a2 = cpml(a2, psi[5], np_, p.tab_h[2][z]);
                    p.psi[8][iz] = np_;
                }
                const float e = a1 + a2;
                float u = Myz * e;
                if (ZM != 0) {
                    float sr = 0.f;
#pragma unroll
                    for (int l = 0; l < R; ++l)
                        if (l < n_mech) {
                            const float n_ = fmaf(p.zen.As[l], r5[l], (p.zen.Bs[l] * gs) * e);
                            sr += r5[l] + n_;
                            p.r[5][l * G + i] = n_;
                        }
                    u = fmaf(0.5f * Myz, sr, u);
                }
                p.s[5][i] = s_yz + u * p.dt;
            }
        }
        if (t + 1 < kTX3S) {
            xshift<ORD>(wy, vy, x + ORD, p.nx, X, yz);
            xshift<ORD>(wz, vz, x + ORD, p.nx, X, yz);
        }
    }
    pdl_trigger();
}

template <int ORD, int ZM, int NS, typename I, bool PAL>
__global__ void __launch_bounds__(kBX3 *kBY3, kStressMinBlocks) k_normal3d(const StepParams p) {
    normal3d_body<ORD, ZM, NS, I, PAL>(p, blockIdx.z);
}

template <int ORD, int ZM, int NS, typename I, bool PAL>
__global__ void __launch_bounds__(kBX3 *kBY3, kStressMinBlocks) k_shear3d(const StepParams p) {
    shear3d_body<ORD, ZM, NS, I, PAL>(p, blockIdx.z);
}

// Both stress updates in one launch: block z-index 2c updates the normal
// stresses of x-chunk c, 2c + 1 its shear stresses.  Both read the same
// velocities at about the same time, so the second read of a chunk mostly
// hits L2, and a step has one launch boundary fewer.
template <int ORD, int ZM, int NS, typename I, bool PAL>
__global__ void __launch_bounds__(kBX3 *kBY3, kStressMinBlocks) k_stress3d(const StepParams p) {
    if (blockIdx.z & 1) shear3d_body<ORD, ZM, NS, I, PAL>(p, blockIdx.z >> 1);
    else normal3d_body<ORD, ZM, NS, I, PAL>(p, blockIdx.z >> 1);
}

// Velocity update, x-marching: thread (z, y) updates TX consecutive nodes
// along x; the x-derivatives of sxx, sxy, sxz come from register windows that
// take one new plane per node, the y- and z-derivatives from loads.
template <int ORD, typename I, int TX>
__global__ void __launch_bounds__(kBX3 *kBY3, kVelocityMinBlocks) k_velocity3d(const StepParams p, const int j) {
    const int z = blockIdx.x * kZB3 + (threadIdx.y % kZW3) * kBX3 + threadIdx.x;
    const int y = blockIdx.y * kYB3 + threadIdx.y / kZW3;
    // x-chunks in reverse launch order with snake_3d: the stress launch before
    // wrote the high chunks last, so they are the ones still in L2
    const int x0 = (p.snake_3d ? gridDim.z - 1 - blockIdx.z : blockIdx.z) * TX;
    const int tid = threadIdx.y * kBX3 + threadIdx.x;
    const int blk = (blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
    const bool col = y < p.ny && z < p.nz;
    const I X = (I)p.plane, Y = (I)p.pitch, yz = (I)y * Y + z;
    const float *__restrict__ sxx = p.s[0];
    const float *__restrict__ syy = p.s[1];
    const float *__restrict__ szz = p.s[2];
    const float *__restrict__ sxy = p.s[3];
    const float *__restrict__ sxz = p.s[4];
    const float *__restrict__ syz = p.s[5];
    const int sy = col ? strip_index(p.strip[1], y) : -1, sz = col ? strip_index(p.strip[2], z) : -1;
    // vz region in (y, z); outside the vz region all three components are zero (wgsl:1754-1758)
    const bool yz_vz = col && y >= ORD && y < p.ny - ORD + 1 && z >= ORD - 1 && z < p.nz - ORD;
    const int q0 = __ldg(p.src_block_start + blk), q1 = __ldg(p.src_block_start + blk + 1);
    // interior sweep (every test compiled out), x-y interior sweep (z tests
    // per lane) or the general sweep; blocks with a source node take the
    // general one
    const bool fast = interior_warp<ORD, TX>(p, y, z, x0, sy, sz) && q0 == q1;
    const bool fast_xy = !fast && q0 == q1 && p.xy_sweep_3d && xy_interior_warp<ORD, TX>(p, y, z, x0, sy);
    if (p.prefetch_3d == 2 && col) {   // velocities (last written two launches back) and dt / rho, every node
#pragma unroll
        for (int t = 0; t < TX; ++t) {
            const int x = x0 + t;
            if (x < p.nx) {
                const I i = (I)x * X + yz;
                prefetch_l2(p.v[0] + i);
                prefetch_l2(p.v[1] + i);
                prefetch_l2(p.v[2] + i);
                prefetch_l2(p.dtw[0] + i);
                prefetch_l2(p.dtw[1] + i);
            }
        }
    }
    pdl_wait();
    if (p.prefetch_3d && col) {   // the later nodes' velocities, dt / rho (mode 1) and stresses
#pragma unroll
        for (int t = 1; t < TX; ++t) {
            const int x = x0 + t;
            if (x < p.nx) {
                const I i = (I)x * X + yz;
                if (p.prefetch_3d == 1) {
                    prefetch_l2(p.v[0] + i);
                    prefetch_l2(p.v[1] + i);
                    prefetch_l2(p.v[2] + i);
                    prefetch_l2(p.dtw[0] + i);
                    prefetch_l2(p.dtw[1] + i);
                }
#pragma unroll
                for (int f = 0; f < 6; ++f) prefetch_l2(p.s[f] + i);
            }
        }
    }
    const int k = *p.step_base + j;
    unsigned vmax = 0u;  // max |v|^2 as float bits (v2 >= 0 or NaN: NaN ranks highest)
    bool bad = false;
    // MODE 2: interior warp; 1: x-y interior warp; 0: general
    auto sweep = [&](auto mode_tag) {
        constexpr int MODE = decltype(mode_tag)::value;
        constexpr bool FAST = MODE == 2, XY = MODE >= 1;
        const int syl = XY ? -1 : sy, szl = FAST ? -1 : sz;
        // sxx planes [x-ORD, x+ORD-1] (vx), sxy and sxz planes [x-ORD+1, x+ORD] (vy, vz)
        float wa[2 * ORD], wb[2 * ORD], wc[2 * ORD];
        xwindow<ORD, !XY>(wa, sxx, x0 - ORD, p.nx, X, yz);
        xwindow<ORD, !XY>(wb, sxy, x0 - ORD + 1, p.nx, X, yz);
        xwindow<ORD, !XY>(wc, sxz, x0 - ORD + 1, p.nx, X, yz);
#pragma unroll
        for (int t = 0; t < TX; ++t) {
            const int x = x0 + t;
            if (!XY && x >= p.nx) break;
            const I i = (I)x * X + yz;
            const bool in_vz = FAST || (yz_vz && (XY || (x >= ORD - 1 && x < p.nx - ORD)));
            const bool in_vx = FAST || (in_vz && (XY || x >= ORD) && z >= ORD);        // vx region within the vz region
            const bool in_vy = FAST || (in_vz && (XY || y < p.ny - ORD) && z >= ORD);  // vy region within the vz region
            const int sx = XY ? -1 : strip_index(p.strip[0], x);
            const I ix = ((I)sx * p.ny + y) * Y + z;
            const I iy = ((I)x * p.strip[1].width + syl) * Y + z;
            const I iz = ((I)x * p.ny + y) * p.strip[2].width + szl;
            // ---- loads ----
            Pairs<ORD> xb, xe, yb, ye, zb, ze;
            float v0[3] = {0.f, 0.f, 0.f};
            float2 dtx = make_float2(0.f, 0.f), dty = make_float2(0.f, 0.f);
            float psi[9] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
            if (in_vx) {
                xb = load_pairs<ORD, false>(sxy, i, Y);
                xe = load_pairs<ORD, false>(sxz, i, (I)1);
                v0[0] = p.v[0][i];
                dtx = __ldg(p.dtw[0] + i);
                if (sx >= 0) psi[0] = p.psi[9][ix];
                if (syl >= 0) psi[1] = p.psi[10][iy];
                if (szl >= 0) psi[2] = p.psi[11][iz];
            }
            if (in_vy) {
                yb = load_pairs<ORD, true>(syy, i, Y);
                ye = load_pairs<ORD, false>(syz, i, (I)1);
                v0[1] = p.v[1][i];
                if (sx >= 0) psi[3] = p.psi[12][ix];
                if (syl >= 0) psi[4] = p.psi[13][iy];
                if (szl >= 0) psi[5] = p.psi[14][iz];
            }
            if (in_vz) {
                zb = load_pairs<ORD, false>(syz, i, Y);
                ze = load_pairs<ORD, true>(szz, i, (I)1);
                v0[2] = p.v[2][i];
                dty = __ldg(p.dtw[1] + i);
                if (sx >= 0) psi[6] = p.psi[15][ix];
                if (syl >= 0) psi[7] = p.psi[16][iy];
                if (szl >= 0) psi[8] = p.psi[17][iz];
            }
            // ---- update ----
            float vxn = 0.f, vyn = 0.f, vzn = 0.f, np_;
            // vx: sxx[x+c]-sxx[x-c-1], sxy[y+c]-sxy[y-c-1], sxz[z+c]-sxz[z-c-1]
            if (in_vx) {
                float a = wderiv<ORD>(wa, p), b = deriv(xb, p, 1), e = deriv(xe, p, 2);
                if (sx >= 0) {
                    a = cpml(a, psi[0], np_, p.tab_f[0][x]);
                    p.psi[9][ix] = np_;
                }
                if (syl >= 0) {
                    b = cpml(b, psi[1], np_, p.tab_f[1][y]);
                    p.psi[10][iy] = np_;
                }
                if (szl >= 0) {
                    e = cpml(e, psi[2], np_, p.tab_f[2][z]);
                    p.psi[11][iz] = np_;
                }
                vxn = wgsl_velocity(v0[0], a + b + e, dtx);
            }
            // vy: sxy[x+c+1]-sxy[x-c], syy[y+c+1]-syy[y-c], syz[z+c]-syz[z-c-1]
            if (in_vy) {
                float a = wderiv<ORD>(wb, p), b = deriv(yb, p, 1), e = deriv(ye, p, 2);
                if (sx >= 0) {
                    a = cpml(a, psi[3], np_, p.tab_h[0][x]);
                    p.psi[12][ix] = np_;
                }
                if (syl >= 0) {
                    b = cpml(b, psi[4], np_, p.tab_h[1][y]);
                    p.psi[13][iy] = np_;
                }
                if (szl >= 0) {
                    e = cpml(e, psi[5], np_, p.tab_f[2][z]);
                    p.psi[14][iz] = np_;
                }
                vyn = wgsl_velocity(v0[1], a + b + e, dty);
            }
            // vz: sxz[x+c+1]-sxz[x-c], syz[y+c]-syz[y-c-1], szz[z+c+1]-szz[z-c]
            if (in_vz) {
                float a = wderiv<ORD>(wc, p), b = deriv(zb, p, 1), e = deriv(ze, p, 2);
                if (sx >= 0) {
                    a = cpml(a, psi[6], np_, p.tab_h[0][x]);
                    p.psi[15][ix] = np_;
                }
                if (syl >= 0) {
                    b = cpml(b, psi[7], np_, p.tab_f[1][y]);
                    p.psi[16][iy] = np_;
                }
                if (szl >= 0) {
                    e = cpml(e, psi[8], np_, p.tab_h[2][z]);
                    p.psi[17][iz] = np_;
                }
                vzn = wgsl_velocity(v0[2], a + b + e, dty);  // the vy-node density (wgsl3d:1748)
            }
            if constexpr (MODE == 0) {
                for (int q = q0; q < q1; ++q) {
                    const Source s = p.src[q];
                    if (s.cell == i && k < p.src_rows)
                        vzn += wgsl_source(__ldg(p.src_tab + (int64_t)k * p.src_ncol + s.col), s.scale, p.dt);
                }
            }
            p.v[0][i] = vxn;
            p.v[1][i] = vyn;
            p.v[2][i] = vzn;
            const float v2 = fmaf(vxn, vxn, fmaf(vyn, vyn, vzn * vzn));
            bad |= !(v2 <= p.v2_threshold);
            vmax = max(vmax, __float_as_uint(v2));
            if (t + 1 < TX) {
                xshift<ORD, !XY>(wa, sxx, x + ORD, p.nx, X, yz);
                xshift<ORD, !XY>(wb, sxy, x + ORD + 1, p.nx, X, yz);
                xshift<ORD, !XY>(wc, sxz, x + ORD + 1, p.nx, X, yz);
            }
        }
    };
    if (fast) sweep(std::integral_constant<int, 2>{});
    else if (fast_xy) {
        if (col) sweep(std::integral_constant<int, 1>{});
    } else if (col && x0 < p.nx) sweep(std::integral_constant<int, 0>{});

    // receivers: global thread g samples receiver g (szz is final for step k)
    const int g = blk * (kBX3 * kBY3) + tid;
    if (g < p.n_rec && k >= __ldg(p.rec_first_step + g) && !(p.rec_chunked && p.rec_chunked[g])) {
        float acc = 0.f;
        for (int q = __ldg(p.rec_start + g); q < __ldg(p.rec_start + g + 1); ++q) acc += fld(szz + __ldg(p.rec_cell + q));
        p.traces[(int64_t)k * p.n_rec + g] = acc;
    }
    warp_stability(__uint_as_float(vmax), bad, reinterpret_cast<unsigned *>(p.block_max) + blk, p.first_bad, k);
    pdl_trigger();
}

template <int ORD, typename I, bool PAL>
void launch_idx(const StepParams &p, int zen_mode, int j, cudaStream_t st, int parts) {
    const dim3 block(kBX3, kBY3);
    const bool three = p.zen.n == 3;
    if (parts & 1) {
        const dim3 grid((p.nz + kZB3 - 1) / kZB3, (p.ny + kYB3 - 1) / kYB3, (p.nx + kTX3S - 1) / kTX3S);
        if (p.stress_pair_3d) {
            const dim3 g2(grid.x, grid.y, 2 * grid.z);
            if (zen_mode == 0) launch_pdl(k_stress3d<ORD, 0, 0, I, PAL>, g2, block, st, p);
            else if (zen_mode == 1 && three) launch_pdl(k_stress3d<ORD, 1, 3, I, PAL>, g2, block, st, p);
            else if (zen_mode == 1) launch_pdl(k_stress3d<ORD, 1, kMaxSls, I, PAL>, g2, block, st, p);
            else if (three) launch_pdl(k_stress3d<ORD, 2, 3, I, PAL>, g2, block, st, p);
            else launch_pdl(k_stress3d<ORD, 2, kMaxSls, I, PAL>, g2, block, st, p);
        } else if (zen_mode == 0) {
            launch_pdl(k_normal3d<ORD, 0, 0, I, PAL>, grid, block, st, p);
            launch_pdl(k_shear3d<ORD, 0, 0, I, PAL>, grid, block, st, p);
        } else if (zen_mode == 1 && three) {
            launch_pdl(k_normal3d<ORD, 1, 3, I, PAL>, grid, block, st, p);
            launch_pdl(k_shear3d<ORD, 1, 3, I, PAL>, grid, block, st, p);
        } else if (zen_mode == 1) {
            launch_pdl(k_normal3d<ORD, 1, kMaxSls, I, PAL>, grid, block, st, p);
            launch_pdl(k_shear3d<ORD, 1, kMaxSls, I, PAL>, grid, block, st, p);
        } else if (three) {
            launch_pdl(k_normal3d<ORD, 2, 3, I, PAL>, grid, block, st, p);
            launch_pdl(k_shear3d<ORD, 2, 3, I, PAL>, grid, block, st, p);
        } else {
            launch_pdl(k_normal3d<ORD, 2, kMaxSls, I, PAL>, grid, block, st, p);
            launch_pdl(k_shear3d<ORD, 2, kMaxSls, I, PAL>, grid, block, st, p);
        }
    }
    if constexpr (!PAL) {   // the velocity kernel has no palette variant
        if (!(parts & 2)) return;
        const dim3 grid((p.nz + kZB3 - 1) / kZB3, (p.ny + kYB3 - 1) / kYB3, (p.nx + p.tx - 1) / p.tx);
        launch_pdl(k_velocity3d<ORD, I, velocity_tx_3d(ORD)>, grid, block, st, p, j);  // p.tx == velocity_tx_3d(ORD)
    }
}

}  // namespace
}  // namespace ts
