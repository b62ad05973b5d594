// Receivers with many points: a parallel, deterministic sum per step.
//
// The step kernels sample a receiver by one thread summing its points
// serially (ts_kernels2d.cuh, ts_kernels3d.cuh), which is right for the
// one-to-few-point elements of linear arrays and receiver planes.  An
// element such as the reference's circular probe (SimulationProbeMonoCirc,
// Simulator3D.py:248-313; 12,645 points in ensaios/ensaio_mono/aco_cfg.json)
// would put thousands of dependent loads on one thread every step.  Those
// receivers ("chunked" ones, more than kChunkedMinPoints points) are split
// into chunks of up to kChunkPoints points; after the velocity kernel of a
// step, k_receiver_chunks sums each chunk in one block (fixed lane order and
// a fixed shuffle tree) into a partial sum, and the last block to finish
// adds every chunked receiver's partials in chunk order into its trace
// (gated by its first recorded step as the inline path is).  The sum order
// is fixed, so results are deterministic; it differs from the serial order
// by rounding only.
#include <cuda_runtime.h>

#include "ts_internal.cuh"

namespace ts {
namespace {

constexpr int kChunkThreads = 256;

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__global__ void __launch_bounds__(kChunkThreads) k_receiver_chunks(const RecChunks rc, const float *field,
                                                                     float *traces, const int *first,
                                                                     const int *step_base, int j, int n_rec) {
    __shared__ float s_warp[kChunkThreads / 32];
    __shared__ int s_last;
    pdl_wait();
    const int k = *step_base + j;
    const int2 ch = rc.chunk[blockIdx.x];   // points [ch.x, ch.y) of the CSR
    float acc = 0.f;
    for (int q = ch.x + (int)threadIdx.x; q < ch.y; q += kChunkThreads) acc += __ldca(field + rc.cell[q]);
    acc = warp_sum(acc);
    if ((threadIdx.x & 31) == 0) s_warp[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x < 32) {
        float v = threadIdx.x < kChunkThreads / 32 ? s_warp[threadIdx.x] : 0.f;
        v = warp_sum(v);
        if (threadIdx.x == 0) {
            rc.partial[blockIdx.x] = v;
            __threadfence();
            s_last = atomicAdd(rc.counter, 1u) == gridDim.x - 1;
        }
    }
    __syncthreads();
    if (s_last) {   // every partial of this step is written and visible
        __threadfence();
        for (int c = threadIdx.x; c < rc.n_chunked; c += kChunkThreads) {
            const int r = rc.receiver[c];
            if (k < first[r]) continue;
            float s = 0.f;
            for (int q = rc.rchunk[c]; q < rc.rchunk[c + 1]; ++q) s += __ldcg(rc.partial + q);
            traces[(int64_t)k * n_rec + r] = s;
        }
        if (threadIdx.x == 0) *rc.counter = 0u;   // for the next step
    }
    pdl_trigger();
}

}  // namespace

void launch_receiver_chunks(const StepParams &p, const RecChunks &rc, int j, cudaStream_t st) {
    if (rc.n_chunks <= 0) return;
    const float *field = p.s[2] ? p.s[2] : p.s[1];   // szz in 3D, syy in 2D (no szz there)
    launch_pdl(k_receiver_chunks, dim3(rc.n_chunks), dim3(kChunkThreads), st, rc, field, p.traces,
               p.rec_first_step, p.step_base, j, p.n_rec);
}

}  // namespace ts
