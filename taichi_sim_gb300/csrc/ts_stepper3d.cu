// 3D staggered-grid (visco)elastic time step on sm_103a.
//
// One time step = k_stress3d (sxx, syy, szz, sxy, sxz, syz with CPML strips
// and the Zener update fused) followed by k_velocity3d (vx, vy, vz with
// CPML, Dirichlet zeroing, source injection, receiver sampling of szz and
// stability bookkeeping fused).  Thread (tx, ty, tz) owns node
// (z = 32 bx + tx, y = 4 by + ty, x = 2 bz + tz): z is the contiguous axis.
//
// Semantics: family TS_WGSL3D, shader_webgpu_3D_viscoelastic.wgsl:1341-1773
// and :1824-1843, including its quirks (normal stresses use point
// rho/cp/cs, shear moduli average rho and cs over 4 nodes without the
// cs == 0 test, vz uses the vy-node density, all three velocities are zeroed
// outside the vz region, the source drives vz).
#include <cuda_runtime.h>
#include "ts_internal.cuh"

namespace ts {
namespace {

__device__ __forceinline__ float cpml_update(float d, float *psi, const Cpml &t) {
    float p = fmaf(t.b, *psi, t.a * d);
    *psi = p;
    return fmaf(d, t.ik, p);
}

struct Idx3 {
    int x, y, z;
    int64_t i;
};

__device__ __forceinline__ float *psi_x(const StepParams &p, int k, int sx, const Idx3 &n) {
    return p.psi[k] + ((int64_t)sx * p.ny + n.y) * p.pitch + n.z;
}
__device__ __forceinline__ float *psi_y(const StepParams &p, int k, int sy, const Idx3 &n) {
    return p.psi[k] + ((int64_t)n.x * p.strip[1].width + sy) * p.pitch + n.z;
}
__device__ __forceinline__ float *psi_z(const StepParams &p, int k, int sz, const Idx3 &n) {
    return p.psi[k] + ((int64_t)n.x * p.ny + n.y) * p.strip[2].width + sz;
}

// x, y and z derivative (forward-staggered "plus" or backward "minus")
template <int ORD, bool PLUS>
__device__ __forceinline__ float dfd(const float *__restrict__ f, int64_t i, int64_t stride, const float *cd) {
    float a = 0.f;
#pragma unroll
    for (int c = 0; c < ORD; ++c) {
        const float hi = __ldg(f + i + (PLUS ? (c + 1) : c) * stride);
        const float lo = __ldg(f + i - (PLUS ? c : (c + 1)) * stride);
        a = fmaf(cd[c], hi - lo, a);
    }
    return a;
}

template <int ZM>
__device__ __forceinline__ float zener_sum(const StepParams &p, int which, int64_t i, float drive, bool p_wave,
                                           float g) {
    float s = 0.f;
#pragma unroll
    for (int l = 0; l < kMaxSls; ++l) {
        if (l >= p.zen.n) break;
        float *rr = p.r[which] + l * p.grid_elems + i;
        const float o = *rr;
        const float A = p_wave ? p.zen.Ap[l] : p.zen.As[l];
        const float B = (p_wave ? p.zen.Bp[l] : p.zen.Bs[l]) * g;
        const float n_ = fmaf(A, o, B * drive);
        s += o + n_;
        *rr = n_;
    }
    return s;
}

template <int ORD, int ZM>
__global__ void __launch_bounds__(kBX3 *kBY3 *kBZ3) k_stress3d(const StepParams p) {
    Idx3 n;
    n.z = blockIdx.x * kBX3 + threadIdx.x;
    n.y = blockIdx.y * kBY3 + threadIdx.y;
    n.x = blockIdx.z * kBZ3 + threadIdx.z;
    if (n.x >= p.nx || n.y >= p.ny || n.z >= p.nz) return;
    const int64_t X = p.plane, Y = p.pitch;
    n.i = n.x * X + n.y * Y + n.z;
    const int64_t i = n.i;
    const int x = n.x, y = n.y, z = n.z;
    const float *vx = p.v[0], *vy = p.v[1], *vz = p.v[2];
    const int sx = strip_index(p.strip[0], x), sy = strip_index(p.strip[1], y), sz = strip_index(p.strip[2], z);
    const float gs = ZM == 2 ? __ldg(p.g_s + i) : 1.f;

    // ---- normal stresses ----
    if (x >= ORD - 1 && x < p.nx - ORD && y >= ORD && y < p.ny - ORD + 1 && z >= ORD && z < p.nz - ORD + 1) {
        float ddx = dfd<ORD, true>(vx, i, X, p.cd[0]);
        float ddy = dfd<ORD, false>(vy, i, Y, p.cd[1]);
        float ddz = dfd<ORD, false>(vz, i, 1, p.cd[2]);
        if (sx >= 0) ddx = cpml_update(ddx, psi_x(p, 0, sx, n), p.tab_h[0][x]);
        if (sy >= 0) ddy = cpml_update(ddy, psi_y(p, 1, sy, n), p.tab_f[1][y]);
        if (sz >= 0) ddz = cpml_update(ddz, psi_z(p, 2, sz, n), p.tab_f[2][z]);
        const float L = __ldg(p.lam_dt + i), M = __ldg(p.mu_dt + i);
        const float L2M = fmaf(2.f, M, L);
        float ux = fmaf(L2M, ddx, L * (ddy + ddz));
        float uy = fmaf(L2M, ddy, L * (ddx + ddz));
        float uz = fmaf(L2M, ddz, L * (ddx + ddy));
        if (ZM != 0) {
            const float gp = ZM == 2 ? __ldg(p.g_p + i) : 1.f;
            const float div = ddx + ddy + ddz;
            const float third = div * (1.f / 3.f);
            const float srxx = zener_sum<ZM>(p, 0, i, div, true, gp);
            const float sryy = zener_sum<ZM>(p, 1, i, ddx - third, false, gs);
            const float srzz = zener_sum<ZM>(p, 2, i, ddy - third, false, gs);
            const float hl23 = 0.5f * fmaf(2.f / 3.f, M, L);
            ux = fmaf(hl23, srxx, fmaf(M, sryy, ux));
            uy = fmaf(hl23, srxx, fmaf(M, srzz, uy));
            uz = fmaf(0.5f * L2M, srxx, fmaf(-M * (1.f / 3.f), sryy + srzz, uz));
        }
        p.s[0][i] += ux;
        p.s[1][i] += uy;
        p.s[2][i] += uz;
    }
    // ---- sigma_xy and sigma_xz: x in [ORD, nx-ORD+1), y, z in [ORD-1, n-ORD) ----
    if (x >= ORD && x < p.nx - ORD + 1 && y >= ORD - 1 && y < p.ny - ORD && z >= ORD - 1 && z < p.nz - ORD) {
        float a1 = dfd<ORD, false>(vy, i, X, p.cd[0]);
        float a2 = dfd<ORD, true>(vx, i, Y, p.cd[1]);
        if (sx >= 0) a1 = cpml_update(a1, psi_x(p, 3, sx, n), p.tab_f[0][x]);
        if (sy >= 0) a2 = cpml_update(a2, psi_y(p, 4, sy, n), p.tab_h[1][y]);
        const float Mxy = __ldg(p.mus_dt[0] + i);
        float u = Mxy * (a1 + a2);
        if (ZM != 0) u = fmaf(0.5f * Mxy, zener_sum<ZM>(p, 3, i, a1 + a2, false, gs), u);
        p.s[3][i] += u;

        float b1 = dfd<ORD, false>(vz, i, X, p.cd[0]);
        float b2 = dfd<ORD, true>(vx, i, 1, p.cd[2]);
        if (sx >= 0) b1 = cpml_update(b1, psi_x(p, 5, sx, n), p.tab_f[0][x]);
        if (sz >= 0) b2 = cpml_update(b2, psi_z(p, 6, sz, n), p.tab_h[2][z]);
        const float Mxz = __ldg(p.mus_dt[1] + i);
        float w = Mxz * (b1 + b2);
        if (ZM != 0) w = fmaf(0.5f * Mxz, zener_sum<ZM>(p, 4, i, b1 + b2, false, gs), w);
        p.s[4][i] += w;
    }
    // ---- sigma_yz: x, y, z in [ORD-1, n-ORD) ----
    if (x >= ORD - 1 && x < p.nx - ORD && y >= ORD - 1 && y < p.ny - ORD && z >= ORD - 1 && z < p.nz - ORD) {
        float a1 = dfd<ORD, true>(vz, i, Y, p.cd[1]);
        float a2 = dfd<ORD, true>(vy, i, 1, p.cd[2]);
        if (sy >= 0) a1 = cpml_update(a1, psi_y(p, 7, sy, n), p.tab_h[1][y]);
        if (sz >= 0) a2 = cpml_update(a2, psi_z(p, 8, sz, n), p.tab_h[2][z]);
        const float Myz = __ldg(p.mus_dt[2] + i);
        float u = Myz * (a1 + a2);
        if (ZM != 0) u = fmaf(0.5f * Myz, zener_sum<ZM>(p, 5, i, a1 + a2, false, gs), u);
        p.s[5][i] += u;
    }
}

template <int ORD>
__global__ void __launch_bounds__(kBX3 *kBY3 *kBZ3) k_velocity3d(const StepParams p, const int j) {
    Idx3 n;
    n.z = blockIdx.x * kBX3 + threadIdx.x;
    n.y = blockIdx.y * kBY3 + threadIdx.y;
    n.x = blockIdx.z * kBZ3 + threadIdx.z;
    const int tid = (threadIdx.z * kBY3 + threadIdx.y) * kBX3 + threadIdx.x;
    const int blk = (blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
    const int k = *p.step_base + j;
    const bool live = n.x < p.nx && n.y < p.ny && n.z < p.nz;
    const int64_t X = p.plane, Y = p.pitch;
    n.i = (int64_t)n.x * X + n.y * Y + n.z;
    const int64_t i = n.i;
    const int x = n.x, y = n.y, z = n.z;
    float v2 = 0.f;

    if (live) {
        const float *sxx = p.s[0], *syy = p.s[1], *szz = p.s[2], *sxy = p.s[3], *sxz = p.s[4], *syz = p.s[5];
        const int sx = strip_index(p.strip[0], x), sy = strip_index(p.strip[1], y), sz = strip_index(p.strip[2], z);
        // vz region; outside it all three components are zero (wgsl:1754-1758)
        const bool in_vz = x >= ORD - 1 && x < p.nx - ORD && y >= ORD && y < p.ny - ORD + 1 && z >= ORD - 1 &&
                           z < p.nz - ORD;
        float vxn = 0.f, vyn = 0.f, vzn = 0.f;
        if (in_vz) {
            const float dtr_y = __ldg(p.dtr[1] + i);
            if (x >= ORD && z >= ORD) {  // vx region within the vz region
                float a = dfd<ORD, false>(sxx, i, X, p.cd[0]);
                float b = dfd<ORD, false>(sxy, i, Y, p.cd[1]);
                float e = dfd<ORD, false>(sxz, i, 1, p.cd[2]);
                if (sx >= 0) a = cpml_update(a, psi_x(p, 9, sx, n), p.tab_f[0][x]);
                if (sy >= 0) b = cpml_update(b, psi_y(p, 10, sy, n), p.tab_f[1][y]);
                if (sz >= 0) e = cpml_update(e, psi_z(p, 11, sz, n), p.tab_f[2][z]);
                vxn = fmaf(a + b + e, __ldg(p.dtr[0] + i), p.v[0][i]);
            }
            if (y < p.ny - ORD && z >= ORD) {  // vy region within the vz region
                float a = dfd<ORD, true>(sxy, i, X, p.cd[0]);
                float b = dfd<ORD, true>(syy, i, Y, p.cd[1]);
                float e = dfd<ORD, false>(syz, i, 1, p.cd[2]);
                if (sx >= 0) a = cpml_update(a, psi_x(p, 12, sx, n), p.tab_h[0][x]);
                if (sy >= 0) b = cpml_update(b, psi_y(p, 13, sy, n), p.tab_h[1][y]);
                if (sz >= 0) e = cpml_update(e, psi_z(p, 14, sz, n), p.tab_f[2][z]);
                vyn = fmaf(a + b + e, dtr_y, p.v[1][i]);
            }
            float a = dfd<ORD, true>(sxz, i, X, p.cd[0]);
            float b = dfd<ORD, false>(syz, i, Y, p.cd[1]);
            float e = dfd<ORD, true>(szz, i, 1, p.cd[2]);
            if (sx >= 0) a = cpml_update(a, psi_x(p, 15, sx, n), p.tab_h[0][x]);
            if (sy >= 0) b = cpml_update(b, psi_y(p, 16, sy, n), p.tab_f[1][y]);
            if (sz >= 0) e = cpml_update(e, psi_z(p, 17, sz, n), p.tab_h[2][z]);
            vzn = fmaf(a + b + e, dtr_y, p.v[2][i]);
        }
        const int q0 = __ldg(p.src_block_start + blk), q1 = __ldg(p.src_block_start + blk + 1);
        for (int q = q0; q < q1; ++q) {
            const Source s = p.src[q];
            if (s.cell == i && k < p.src_rows) vzn = fmaf(__ldg(p.src_tab + (int64_t)k * p.src_ncol + s.col), s.scale, vzn);
        }
        p.v[0][i] = vxn;
        p.v[1][i] = vyn;
        p.v[2][i] = vzn;
        v2 = fmaf(vxn, vxn, fmaf(vyn, vyn, vzn * vzn));
    }

    const int g = blk * (kBX3 * kBY3 * kBZ3) + tid;
    if (g < p.n_rec && k >= __ldg(p.rec_first_step + g)) {
        float acc = 0.f;
        for (int q = __ldg(p.rec_start + g); q < __ldg(p.rec_start + g + 1); ++q) acc += p.s[2][__ldg(p.rec_cell + q)];
        p.traces[(int64_t)k * p.n_rec + g] = acc;
    }

    const bool bad = live && !(v2 <= p.v2_threshold);
    unsigned m = __reduce_max_sync(0xffffffffu, __float_as_uint(v2));
    __shared__ unsigned wmax[kBX3 * kBY3 * kBZ3 / 32];
    if ((tid & 31) == 0) wmax[tid >> 5] = m;
    const int any_bad = __syncthreads_or(bad);
    if (tid == 0) {
        unsigned bm = wmax[0];
#pragma unroll
        for (int w = 1; w < kBX3 * kBY3 * kBZ3 / 32; ++w) bm = max(bm, wmax[w]);
        unsigned *slot = reinterpret_cast<unsigned *>(p.block_max) + blk;
        *slot = max(*slot, bm);
        if (any_bad) atomicMin(p.first_bad, k);
    }
}

template <int ORD>
void launch_ord(const StepParams &p, int zen_mode, int j, cudaStream_t st, int parts) {
    dim3 block(kBX3, kBY3, kBZ3);
    dim3 grid((p.nz + kBX3 - 1) / kBX3, (p.ny + kBY3 - 1) / kBY3, (p.nx + kBZ3 - 1) / kBZ3);
    if (parts & 1) {
        if (zen_mode == 0) k_stress3d<ORD, 0><<<grid, block, 0, st>>>(p);
        else if (zen_mode == 1) k_stress3d<ORD, 1><<<grid, block, 0, st>>>(p);
        else k_stress3d<ORD, 2><<<grid, block, 0, st>>>(p);
    }
    if (parts & 2) k_velocity3d<ORD><<<grid, block, 0, st>>>(p, j);
}

}  // namespace

int blocks_3d(const StepParams &p) {
    return ((p.nz + kBX3 - 1) / kBX3) * ((p.ny + kBY3 - 1) / kBY3) * ((p.nx + kBZ3 - 1) / kBZ3);
}

void launch_step_3d(const StepParams &p, int ord, int zen_mode, int j, cudaStream_t st, int parts) {
    switch (ord) {
    case 2: launch_ord<2>(p, zen_mode, j, st, parts); break;
    case 3: launch_ord<3>(p, zen_mode, j, st, parts); break;
    case 4: launch_ord<4>(p, zen_mode, j, st, parts); break;
    case 5: launch_ord<5>(p, zen_mode, j, st, parts); break;
    case 6: launch_ord<6>(p, zen_mode, j, st, parts); break;
    default: break;
    }
}

}  // namespace ts
