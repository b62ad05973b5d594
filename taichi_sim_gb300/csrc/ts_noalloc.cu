// Allocation-free 2D elastic stepper: ts_run_noalloc_2d.
//
// Some callers cannot call cudaMalloc: an application that hands this code
// only buffers from its own pre-sized device-memory pool, a serving process
// whose memory budget is fixed at start-up, or a time-critical loop that
// cannot afford an allocation's latency and implicit synchronisation.  This
// entry point serves them: it advances a 2D elastic simulation (the WGSL
// backend's semantics, shader_webgpu_viscoelastic.wgsl:829-1072 with
// viscoelastic_attn = 0) in buffers the caller owns, and keeps its only
// scratch - the eight CPML convolution memories, one full grid each, as in
// the reference - in a file-scope device array of fixed size.  It calls no
// cudaMalloc, cudaFree or other allocating routine.
//
// The array holds TS_NOALLOC_SCRATCH_FLOATS floats (32 MiB): grids of at
// most TS_NOALLOC_SCRATCH_FLOATS / 8 = 1,048,576 nodes.  Every GPU that loads
// this library keeps it until the process exits.  All calls share it and it
// keeps the last call's contents: a call with step0 == 0 clears it (a new
// simulation), a call with step0 > 0 continues from what the previous call
// left, so calls that overlap on the GPU, or interleave two simulations,
// race on it.  The host needs the array's device address, which is looked up
// (cudaGetSymbolAddress) by the first call on each device; make that first
// call before any stream capture.  The looked-up address is kept for the
// life of the process: it does not survive a reset of the device's context
// (cudaDeviceReset), after which this entry point must not be called.
//
// Source and receiver cells come as device tables the host cannot read, so
// the kernel range-checks them: entries outside the grid are ignored.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "../../include/taichi_sim_gb300.h"

namespace {

static __device__ __align__(256) float g_noalloc_scratch[TS_NOALLOC_SCRATCH_FLOATS];

constexpr int kMaxDevices = 64;
float *g_scratch_addr[kMaxDevices] = {};
std::mutex g_scratch_mutex;
thread_local std::string g_noalloc_error;

constexpr int kBX = 32, kBY = 8;

struct NaParams {
    int nx, ny, ord;
    float cdx[6], cdy[6];
    float dt;
    float *vx, *vy, *sxx, *syy, *sxy;
    const float *rho, *cp, *cs;
    const float *a_x, *b_x, *k_x, *a_xh, *b_xh, *k_xh;
    const float *a_y, *b_y, *k_y, *a_yh, *b_yh, *k_yh;
    float *psi;  // scratch: 8 grids
    int n_src, n_rec, n_rows;
    const int32_t *src_cell, *rec_cell, *rec_first_step;
    const float *src_value;
    float *traces;
};

__device__ __forceinline__ float at(const float *a, const NaParams &p, int x, int y) {
    return (x < 0 || x >= p.nx || y < 0 || y >= p.ny) ? 0.f : a[(int64_t)x * p.ny + y];
}

__device__ __forceinline__ float conv(float d, float *psi, float a, float b, float k) {
    const float q = fmaf(b, *psi, a * d);
    *psi = q;
    return d / k + q;
}

__global__ void k_na_stress(const NaParams p) {
    const int y = blockIdx.x * kBX + threadIdx.x, x = blockIdx.y * kBY + threadIdx.y;
    if (x >= p.nx || y >= p.ny) return;
    const int ord = p.ord, off = ord - 1;
    const int64_t n = (int64_t)p.nx * p.ny, i = (int64_t)x * p.ny + y;
    if (x >= ord - 1 && x < p.nx - ord && y >= ord && y < p.ny - ord + 1) {
        float ddx = 0.f, ddy = 0.f;
        for (int c = 0; c < ord; ++c) {
            ddx = fmaf(p.cdx[c], p.vx[i + (int64_t)(c + 1) * p.ny] - p.vx[i - (int64_t)c * p.ny], ddx);
            ddy = fmaf(p.cdy[c], p.vy[i + c] - p.vy[i - c - 1], ddy);
        }
        ddx = conv(ddx, p.psi + 0 * n + i, p.a_xh[x - off], p.b_xh[x - off], p.k_xh[x - off]);
        ddy = conv(ddy, p.psi + 1 * n + i, p.a_y[y - off], p.b_y[y - off], p.k_y[y - off]);
        const float rh = 0.5f * (at(p.rho, p, x + 1, y) + at(p.rho, p, x, y));
        const float cph = 0.5f * (at(p.cp, p, x + 1, y) + at(p.cp, p, x, y));
        const float c1 = at(p.cs, p, x + 1, y), c0 = at(p.cs, p, x, y);
        const float csl = 0.5f * (c1 + c0);
        const float csm = fminf(c1, c0) == 0.f ? 0.f : csl;
        const float lam = rh * (cph * cph - 2.f * csl * csl), mu = rh * (csm * csm);
        const float l2m = lam + 2.f * mu;
        p.sxx[i] += (l2m * ddx + lam * ddy) * p.dt;
        p.syy[i] += (lam * ddx + l2m * ddy) * p.dt;
    }
    if (x >= ord && x < p.nx - ord + 1 && y >= ord - 1 && y < p.ny - ord) {
        float a = 0.f, b = 0.f;
        for (int c = 0; c < ord; ++c) {
            a = fmaf(p.cdx[c], p.vy[i + (int64_t)c * p.ny] - p.vy[i - (int64_t)(c + 1) * p.ny], a);
            b = fmaf(p.cdy[c], p.vx[i + c + 1] - p.vx[i - c], b);
        }
        a = conv(a, p.psi + 2 * n + i, p.a_x[x - off], p.b_x[x - off], p.k_x[x - off]);
        b = conv(b, p.psi + 3 * n + i, p.a_yh[y - off], p.b_yh[y - off], p.k_yh[y - off]);
        const float rh = 0.5f * (at(p.rho, p, x, y + 1) + at(p.rho, p, x, y));
        const float s1 = at(p.cs, p, x, y + 1), s0 = at(p.cs, p, x, y);
        const float csh = fminf(s1, s0) == 0.f ? 0.f : 0.5f * (s1 + s0);
        p.sxy[i] += (b + a) * (rh * (csh * csh)) * p.dt;
    }
}

__global__ void k_na_velocity(const NaParams p) {
    const int y = blockIdx.x * kBX + threadIdx.x, x = blockIdx.y * kBY + threadIdx.y;
    if (x >= p.nx || y >= p.ny) return;
    const int ord = p.ord, off = ord - 1;
    const int64_t n = (int64_t)p.nx * p.ny, i = (int64_t)x * p.ny + y;
    const bool in_vy = x >= ord - 1 && x < p.nx - ord && y >= ord - 1 && y < p.ny - ord;
    if (!in_vy) {  // the WGSL kernel zeroes both components outside the vy region
        p.vx[i] = 0.f;
        p.vy[i] = 0.f;
        return;
    }
    if (x >= ord && y >= ord) {
        float a = 0.f, b = 0.f;
        for (int c = 0; c < ord; ++c) {
            a = fmaf(p.cdx[c], p.sxx[i + (int64_t)c * p.ny] - p.sxx[i - (int64_t)(c + 1) * p.ny], a);
            b = fmaf(p.cdy[c], p.sxy[i + c] - p.sxy[i - c - 1], b);
        }
        a = conv(a, p.psi + 4 * n + i, p.a_x[x - off], p.b_x[x - off], p.k_x[x - off]);
        b = conv(b, p.psi + 5 * n + i, p.a_y[y - off], p.b_y[y - off], p.k_y[y - off]);
        const float r = p.rho[i];
        if (r > 0.f) p.vx[i] += (a + b) * p.dt / r;
    }
    float a = 0.f, b = 0.f;
    for (int c = 0; c < ord; ++c) {
        a = fmaf(p.cdx[c], p.sxy[i + (int64_t)(c + 1) * p.ny] - p.sxy[i - (int64_t)c * p.ny], a);
        b = fmaf(p.cdy[c], p.syy[i + c + 1] - p.syy[i - c], b);
    }
    a = conv(a, p.psi + 6 * n + i, p.a_xh[x - off], p.b_xh[x - off], p.k_xh[x - off]);
    b = conv(b, p.psi + 7 * n + i, p.a_yh[y - off], p.b_yh[y - off], p.k_yh[y - off]);
    const float r4 = 0.25f * (at(p.rho, p, x, y) + at(p.rho, p, x + 1, y) + at(p.rho, p, x + 1, y + 1) + at(p.rho, p, x, y + 1));
    if (r4 > 0.f) p.vy[i] += (a + b) * p.dt / r4;
}

// Source injection (after the velocity update, as wgsl:1059-1065) and
// receiver sampling of syy (wgsl:1118-1134, one node per receiver).  The
// cell tables live in device memory, where the host cannot check them, so
// the kernel does: a source or receiver whose cell lies outside [0, nx*ny)
// is skipped (its trace row entries are left untouched).  Sources add with
// atomicAdd, so several entries naming one cell all inject.
__global__ void k_na_sources_receivers(const NaParams p, int k) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t n = (int64_t)p.nx * p.ny;
    if (t < p.n_src) {
        const int64_t c = p.src_cell[t];
        if (c >= 0 && c < n) {
            const int x = (int)(c / p.ny), y = (int)(c % p.ny);
            const float r4 = 0.25f * (at(p.rho, p, x, y) + at(p.rho, p, x + 1, y) + at(p.rho, p, x + 1, y + 1) +
                                      at(p.rho, p, x, y + 1));
            if (r4 > 0.f) atomicAdd(p.vy + c, p.src_value[(int64_t)k * p.n_src + t] * p.dt / r4);
        }
    }
    if (t < p.n_rec && k >= p.rec_first_step[t]) {
        const int64_t c = p.rec_cell[t];
        if (c >= 0 && c < n) p.traces[(int64_t)k * p.n_rec + t] = p.syy[c];
    }
}

int na_fail(const std::string &msg) {
    g_noalloc_error = msg;
    return TS_E_ARG;
}

}  // namespace

extern "C" int ts_run_noalloc_2d(const ts_noalloc2d_args *a, void *stream) {
    if (!a) return na_fail("null arguments");
    if (a->ord < 2 || a->ord > 6) return na_fail("ord must be in [2, 6]");
    if (a->nx < 2 * a->ord + 1 || a->ny < 2 * a->ord + 1) return na_fail("grid smaller than the stencil");
    const int64_t cells = (int64_t)a->nx * a->ny;
    if (cells * 8 > (int64_t)TS_NOALLOC_SCRATCH_FLOATS)
        return na_fail("grid of " + std::to_string(cells) + " nodes exceeds the no-allocation scratch (at most " +
                       std::to_string(TS_NOALLOC_SCRATCH_FLOATS / 8) + " nodes)");
    if (!a->vx || !a->vy || !a->sxx || !a->syy || !a->sxy || !a->rho || !a->cp || !a->cs)
        return na_fail("missing field or material buffer");
    if (!a->a_x || !a->b_x || !a->k_x || !a->a_xh || !a->b_xh || !a->k_xh || !a->a_y || !a->b_y || !a->k_y ||
        !a->a_yh || !a->b_yh || !a->k_yh)
        return na_fail("missing CPML table");
    if (a->step0 < 0 || a->n_steps < 0 || (int64_t)a->step0 + a->n_steps > a->n_rows)
        return na_fail("steps beyond the source/trace rows");
    if (a->n_src < 0 || (a->n_src > 0 && (!a->src_cell || !a->src_value))) return na_fail("bad source list");
    if (a->n_rec < 0 || (a->n_rec > 0 && (!a->rec_cell || !a->rec_first_step || !a->traces)))
        return na_fail("bad receiver list");
    if (!(a->dx > 0.f) || !(a->dy > 0.f) || !(a->dt > 0.f)) return na_fail("grid and time steps must be positive");

    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return (g_noalloc_error = cudaGetErrorString(e), TS_E_CUDA);
    if (dev < 0 || dev >= kMaxDevices) return na_fail("device index out of range");
    float *scratch = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_scratch_mutex);
        if (!g_scratch_addr[dev]) {
            void *ptr = nullptr;
            e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
            if (e != cudaSuccess) return (g_noalloc_error = std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e), TS_E_CUDA);
            g_scratch_addr[dev] = static_cast<float *>(ptr);
        }
        scratch = g_scratch_addr[dev];
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);

    NaParams p{};
    p.nx = a->nx;
    p.ny = a->ny;
    p.ord = a->ord;
    for (int c = 0; c < 6; ++c) {
        p.cdx[c] = c < a->ord ? a->coefs[c] / a->dx : 0.f;
        p.cdy[c] = c < a->ord ? a->coefs[c] / a->dy : 0.f;
    }
    p.dt = a->dt;
    p.vx = a->vx;
    p.vy = a->vy;
    p.sxx = a->sxx;
    p.syy = a->syy;
    p.sxy = a->sxy;
    p.rho = a->rho;
    p.cp = a->cp;
    p.cs = a->cs;
    p.a_x = a->a_x; p.b_x = a->b_x; p.k_x = a->k_x;
    p.a_xh = a->a_xh; p.b_xh = a->b_xh; p.k_xh = a->k_xh;
    p.a_y = a->a_y; p.b_y = a->b_y; p.k_y = a->k_y;
    p.a_yh = a->a_yh; p.b_yh = a->b_yh; p.k_yh = a->k_yh;
    p.psi = scratch;
    p.n_src = a->n_src;
    p.n_rec = a->n_rec;
    p.n_rows = a->n_rows;
    p.src_cell = a->src_cell;
    p.src_value = a->src_value;
    p.rec_cell = a->rec_cell;
    p.rec_first_step = a->rec_first_step;
    p.traces = a->traces;

    if (a->step0 == 0) {  // a new simulation: the CPML memories start at zero
        e = cudaMemsetAsync(scratch, 0, (size_t)cells * 8 * sizeof(float), st);
        if (e != cudaSuccess) return (g_noalloc_error = std::string("cudaMemsetAsync: ") + cudaGetErrorString(e), TS_E_CUDA);
    }
    const dim3 block(kBX, kBY), grid((a->ny + kBX - 1) / kBX, (a->nx + kBY - 1) / kBY);
    const int extra = a->n_src > a->n_rec ? a->n_src : a->n_rec;
    for (int j = 0; j < a->n_steps; ++j) {
        k_na_stress<<<grid, block, 0, st>>>(p);
        k_na_velocity<<<grid, block, 0, st>>>(p);
        if (extra > 0) k_na_sources_receivers<<<(extra + 127) / 128, 128, 0, st>>>(p, a->step0 + j);
    }
    e = cudaGetLastError();
    if (e != cudaSuccess) return (g_noalloc_error = std::string("launch: ") + cudaGetErrorString(e), TS_E_CUDA);
    return TS_OK;
}

extern "C" const char *ts_noalloc_last_error(void) { return g_noalloc_error.c_str(); }
