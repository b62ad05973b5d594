// C ABI of the GB300 stepper (include/taichi_sim_gb300.h): validation,
// host-side preparation of the device layout, allocation, the CUDA-graph
// step loop and readback.
//
// Preparation turns the reference's tables into the layout the kernels
// stream (see ts_internal.cuh):
//  * material: per-node moduli and inverse densities with the reference's
//    averaging (sim_taichi_elastic.py:171-178, 223-227, 263, 293;
//    shader_webgpu_viscoelastic.wgsl:863-868, 948-950, 1020, 1032;
//    shader_webgpu_3D_viscoelastic.wgsl:1384-1388, 1481-1483, 1542-1544,
//    1599-1601, 1676, 1690), folded with dt;
//  * Zener constants evaluated like the shaders (wgsl:881-894) and folded
//    into r' = A r + B d;
//  * CPML tables re-indexed by grid node, strips found from where they
//    differ from the identity;
//  * sources: one entry per source node with the value table the reference
//    would read at each step (Taichi: source_term[it-1, idx],
//    sim_taichi_elastic.py:299; WGSL: flat[it * n_src + idx] when
//    idx < n_src, wgsl:67-71), dropped where the reference cannot inject
//    (rho <= 0, or outside the vy region in the Taichi kernel);
//  * receivers: CSR lists of nodes; Taichi records row it-1 for 1-based
//    it >= delay and only inside the normal-stress region
//    (sim_taichi_elastic.py:188-190), WGSL row it for 0-based it >= delay
//    over info_rec_pt (wgsl:1118-1134).
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <utility>
#include <vector>

#include "../../include/taichi_sim_gb300.h"
#include "ts_internal.cuh"
#include "ts_prep.h"

namespace ts {

__global__ void k_advance(int *step_base, int n) {
    if (threadIdx.x == 0 && blockIdx.x == 0) *step_base += n;
}

void launch_advance(int *step_base, int n, cudaStream_t st) { k_advance<<<1, 32, 0, st>>>(step_base, n); }

__global__ void k_reset_scalars(int *first_bad, int *step_base) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        *first_bad = 0x7fffffff;
        *step_base = 0;
    }
}

void launch_reset_scalars(int *first_bad, int *step_base, cudaStream_t st) {
    k_reset_scalars<<<1, 32, 0, st>>>(first_bad, step_base);
}

}  // namespace ts

using ts::Cpml;
using ts::Source;
using ts::StepParams;
using ts::Strip;

namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string &msg) {
    g_last_error = msg;
    return code;
}

int cuda_fail(cudaError_t e, const char *what) {
    g_last_error = std::string(what) + ": " + cudaGetErrorString(e);
    return TS_E_CUDA;
}

#define TS_CUDA(call)                                                   \
    do {                                                                \
        cudaError_t _e = (call);                                        \
        if (_e != cudaSuccess) return cuda_fail(_e, #call);             \
    } while (0)

constexpr int kGraphSteps = 32;

// f(x) for x in [0, n) on up to 16 host threads (rows of the host-side
// preparation; every x writes its own nodes).
template <typename F>
void parallel_rows(int n, const F &f) {
    const unsigned hw = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    const int nt = (int)std::min<int64_t>(hw, std::max(1, n / 4));
    if (nt <= 1) {
        for (int x = 0; x < n; ++x) f(x);
        return;
    }
    std::atomic<int> next{0};
    std::vector<std::thread> pool;
    for (int t = 0; t < nt; ++t)
        pool.emplace_back([&] {
            for (int x; (x = next.fetch_add(1)) < n;) f(x);
        });
    for (auto &t : pool) t.join();
}

// Host tables of the size of a grid, filled by parallel loops: elements
// are left uninitialised by the vector (std::allocator would zero 67 MB per
// 256^3 table on one thread) and written by fill() or by the loops.
template <typename T>
struct NoInitAlloc : std::allocator<T> {
    template <typename U>
    struct rebind {
        using other = NoInitAlloc<U>;
    };
    NoInitAlloc() = default;
    template <typename U>
    NoInitAlloc(const NoInitAlloc<U> &) {}
    template <typename U>
    void construct(U *) noexcept {}
    template <typename U, typename... Args>
    void construct(U *q, Args &&...args) {
        ::new (static_cast<void *>(q)) U(std::forward<Args>(args)...);
    }
};
using hvec = std::vector<float, NoInitAlloc<float>>;

hvec filled(size_t n, float v) {
    hvec out(n);
    constexpr size_t kPart = (size_t)1 << 20;
    const int parts = (int)((n + kPart - 1) / kPart);
    parallel_rows(parts, [&](int q) { std::fill(out.begin() + q * kPart, out.begin() + std::min(n, (q + 1) * kPart), v); });
    return out;
}

// Copies between pageable host memory and the device through a pinned
// staging buffer shared by the process (allocated on first use, kept until
// exit): pageable copies run at a few GB/s, pinned ones at the link's rate.
// Two halves, so the DMA of one chunk overlaps the host copy of the other.
// Small copies go directly.
constexpr size_t kStageHalf = (size_t)16 << 20;
constexpr size_t kStageMin = (size_t)4 << 20;
std::mutex g_stage_mutex;
char *g_stage = nullptr;
cudaEvent_t g_stage_ev[2] = {nullptr, nullptr};

// Host copy of one staging chunk on up to 8 threads (one thread's memcpy
// runs well below the host memory bandwidth).
void host_copy(void *dst, const void *src, size_t bytes) {
    constexpr size_t kPart = (size_t)2 << 20;
    const int parts = (int)std::min<size_t>(8, (bytes + kPart - 1) / kPart);
    if (parts <= 1) {
        std::memcpy(dst, src, bytes);
        return;
    }
    const size_t per = (bytes + parts - 1) / parts;
    std::vector<std::thread> pool;
    for (int t = 1; t < parts; ++t)
        pool.emplace_back([=] {
            const size_t o = t * per;
            if (o < bytes) std::memcpy(static_cast<char *>(dst) + o, static_cast<const char *>(src) + o, std::min(per, bytes - o));
        });
    std::memcpy(dst, src, std::min(per, bytes));
    for (auto &th : pool) th.join();
}

cudaError_t stage_init() {
    if (g_stage) return cudaSuccess;
    cudaError_t e = cudaMallocHost(reinterpret_cast<void **>(&g_stage), 2 * kStageHalf);
    if (e != cudaSuccess) {
        g_stage = nullptr;
        return e;
    }
    for (auto &ev : g_stage_ev)
        if ((e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming)) != cudaSuccess) return e;
    return cudaSuccess;
}

// `rows` rows of `width` bytes: device rows `dpitch` bytes apart, host rows contiguous.
cudaError_t stage_d2h(void *dst, const void *src, size_t width, size_t dpitch, size_t rows, cudaStream_t st) {
    if (width * rows < kStageMin || width > kStageHalf) {
        cudaError_t e = cudaMemcpy2DAsync(dst, width, src, dpitch, width, rows, cudaMemcpyDeviceToHost, st);
        return e != cudaSuccess ? e : cudaStreamSynchronize(st);
    }
    std::lock_guard<std::mutex> lock(g_stage_mutex);
    cudaError_t e = stage_init();
    if (e != cudaSuccess) return e;
    const size_t per = kStageHalf / width, chunks = (rows + per - 1) / per;
    for (size_t c = 0; c <= chunks; ++c) {
        if (c < chunks) {
            const size_t r0 = c * per, n = std::min(per, rows - r0);
            char *buf = g_stage + (c & 1) * kStageHalf;
            if ((e = cudaMemcpy2DAsync(buf, width, static_cast<const char *>(src) + r0 * dpitch, dpitch, width, n,
                                       cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
                (e = cudaEventRecord(g_stage_ev[c & 1], st)) != cudaSuccess)
                return e;
        }
        if (c > 0) {   // the previous chunk: wait for its DMA, copy it out
            const size_t q = c - 1, r0 = q * per, n = std::min(per, rows - r0);
            if ((e = cudaEventSynchronize(g_stage_ev[q & 1])) != cudaSuccess) return e;
            host_copy(static_cast<char *>(dst) + r0 * width, g_stage + (q & 1) * kStageHalf, n * width);
        }
    }
    return cudaSuccess;
}

cudaError_t stage_h2d(void *dst, const void *src, size_t bytes, cudaStream_t st) {
    if (bytes < kStageMin) {
        cudaError_t e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st);
        return e != cudaSuccess ? e : cudaStreamSynchronize(st);
    }
    std::lock_guard<std::mutex> lock(g_stage_mutex);
    cudaError_t e = stage_init();
    if (e != cudaSuccess) return e;
    const size_t chunks = (bytes + kStageHalf - 1) / kStageHalf;
    for (size_t c = 0; c < chunks; ++c) {
        const size_t off = c * kStageHalf, n = std::min(kStageHalf, bytes - off);
        char *buf = g_stage + (c & 1) * kStageHalf;
        if (c >= 2 && (e = cudaEventSynchronize(g_stage_ev[c & 1])) != cudaSuccess) return e;   // half free again
        host_copy(buf, static_cast<const char *>(src) + off, n);
        if ((e = cudaMemcpyAsync(static_cast<char *>(dst) + off, buf, n, cudaMemcpyHostToDevice, st)) != cudaSuccess ||
            (e = cudaEventRecord(g_stage_ev[c & 1], st)) != cudaSuccess)
            return e;
    }
    return cudaStreamSynchronize(st);
}

// Phase times of ts_create on stderr when TS_CREATE_TIMING=1 (diagnostic).
struct PhaseClock {
    bool on = false;
    std::chrono::steady_clock::time_point t0;
    PhaseClock() {
        const char *e = getenv("TS_CREATE_TIMING");
        on = e && e[0] == '1';
        t0 = std::chrono::steady_clock::now();
    }
    void mark(const char *what) {
        if (!on) return;
        const auto t = std::chrono::steady_clock::now();
        fprintf(stderr, "ts_create %-14s %8.3f ms\n", what, std::chrono::duration<double, std::milli>(t - t0).count());
        t0 = t;
    }
};

}  // namespace

struct ts_sim {
    int family = 0, dims = 2, ord = 2, zen_mode = 0;
    int nx = 0, ny = 0, nz = 1, pitch = 0;
    int64_t grid_elems = 0;
    int n_rows = 0, n_rec = 0, n_blocks = 0;
    int steps_done = 0;
    int64_t launches = 0;
    int64_t h2d_bytes = 0, d2h_bytes = 0;
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
    cudaGraphExec_t graph = nullptr;
    std::vector<void *> allocs;
    float *field[9] = {};
    float *traces = nullptr;
    float *block_max = nullptr;
    int *first_bad = nullptr;
    int *step_base = nullptr;
    float *src_tab = nullptr;
    // host copies needed to rebuild the source table
    int src_rows = 0, src_cols_in = 0, n_src_el = 0;
    std::vector<int> src_col_idx;  // reference column of each device column
    std::vector<size_t> state_bytes;
    std::vector<void *> state_ptrs;
    StepParams p{};
    // persistent path (2D elastic, order 2; ts_persist2d.cu)
    ts::RecChunks rc{};   // receivers with many points (stepped path)
    int persist = 0, p_rows = 0, p_blocks = 0, p_threads = 0;
    size_t p_smem = 0;
    ts::PersistArgs pa{};

    template <typename T>
    int alloc(T **ptr, size_t count, bool state) {
        void *d = nullptr;
        size_t bytes = std::max<size_t>(count, 1) * sizeof(T);
        cudaError_t e = cudaMalloc(&d, bytes);
        if (e != cudaSuccess) {
            g_last_error = std::string("cudaMalloc of ") + std::to_string(bytes) + " bytes: " + cudaGetErrorString(e);
            return TS_E_NOMEM;
        }
        allocs.push_back(d);
        *ptr = static_cast<T *>(d);
        if (state) {
            state_ptrs.push_back(d);
            state_bytes.push_back(bytes);
        }
        return TS_OK;
    }

    template <typename T, typename A>
    int upload(T **ptr, const std::vector<T, A> &h) {
        int rc = alloc(ptr, h.size(), false);
        if (rc) return rc;
        if (!h.empty()) TS_CUDA(stage_h2d(*ptr, h.data(), h.size() * sizeof(T), nullptr));
        h2d_bytes += (int64_t)(h.size() * sizeof(T));
        return TS_OK;
    }

    // padded index of grid node (x, y[, z])
    int64_t at(int x, int y, int z = 0) const {
        return dims == 2 ? (int64_t)x * pitch + y : ((int64_t)x * ny + y) * pitch + z;
    }
};

using ts::Axis;

int ts::nodes_per_thread_2d(int64_t cells) {
    if (const char *env = getenv("TS_2D_NODES_PER_THREAD")) {
        const int v = atoi(env);
        if (v == 1 || v == 2 || v == 4) return v;
    }
    return cells >= 800000 ? 2 : 1;
}

// Coefficient palette of a 3D model (and of the 2D order-2 WGSL stepper):
// the distinct tuples of the stress kernels' per-node coefficients (compared
// bit for bit) and each node's 16-bit index into them, numbered in the order
// of first occurrence.  Models built from a few materials (layers,
// inclusions) have a few dozen tuples; false when there are more than 65536
// (the arrays are used).  The grid is scanned in `rows` slabs in parallel
// (each slab's own distinct tuples), then the slabs' tuples are numbered in
// slab order, which is the sequential scan's numbering.
struct PalKey {
    uint32_t w[7];
    bool operator==(const PalKey &o) const { return std::memcmp(w, o.w, sizeof w) == 0; }
};
struct PalHash {
    size_t operator()(const PalKey &k) const {
        uint64_t h = 1469598103934665603ull;   // FNV-1a over the words
        for (uint32_t v : k.w) h = (h ^ v) * 1099511628211ull;
        return (size_t)h;
    }
};

bool build_palette_3d(const hvec *const (&c)[7], int rows, std::vector<uint16_t> &idx,
                      std::vector<ts::Pal3> &table) {
    const size_t n = c[0]->size();
    const size_t per = (n + rows - 1) / rows;
    idx.assign(n, 0);
    table.clear();
    std::vector<std::vector<PalKey>> keys(rows);   // each slab's distinct tuples, first occurrence first
    std::atomic<bool> over{false};
    parallel_rows(rows, [&](int r) {
        std::unordered_map<PalKey, uint16_t, PalHash> ids;
        PalKey last{};
        int last_id = -1;
        for (size_t i = r * per; i < std::min(n, (r + 1) * per); ++i) {
            PalKey k;
            for (int f = 0; f < 7; ++f) std::memcpy(&k.w[f], &(*c[f])[i], 4);
            if (last_id >= 0 && k == last) {   // runs along the last axis share a tuple
                idx[i] = (uint16_t)last_id;
                continue;
            }
            auto it = ids.find(k);
            int id;
            if (it != ids.end()) {
                id = it->second;
            } else {
                if (keys[r].size() == 65536) {
                    over = true;
                    return;
                }
                id = (int)keys[r].size();
                ids.emplace(k, (uint16_t)id);
                keys[r].push_back(k);
            }
            idx[i] = (uint16_t)id;
            last = k;
            last_id = id;
        }
    });
    if (over) return false;
    std::unordered_map<PalKey, uint16_t, PalHash> global;
    std::vector<std::vector<uint16_t>> to_global(rows);
    for (int r = 0; r < rows; ++r)
        for (const PalKey &k : keys[r]) {
            auto it = global.find(k);
            if (it == global.end()) {
                if (table.size() == 65536) return false;
                it = global.emplace(k, (uint16_t)table.size()).first;
                float v[7];
                std::memcpy(v, k.w, sizeof v);
                table.push_back(ts::Pal3{make_float4(v[0], v[1], v[2], v[3]), make_float4(v[4], v[5], v[6], v[3])});
            }
            to_global[r].push_back(it->second);
        }
    parallel_rows(rows, [&](int r) {
        for (size_t i = r * per; i < std::min(n, (r + 1) * per); ++i) idx[i] = to_global[r][idx[i]];
    });
    return true;
}

// dt / rho as a pair (hi, lo), computed in double from the float dt and rho
// (0 where rho <= 0: no update)
static float2 dt_over_rho(float dt, float rho) {
    if (!(rho > 0.f)) return make_float2(0.f, 0.f);
    const double q = (double)dt / (double)rho;
    const float hi = (float)q;
    return make_float2(hi, (float)(q - (double)hi));
}
using ts::make_axis;
using ts::round_up;

// Kernel launches of one time step: 2D stress + velocity; 3D normal stress,
// shear stress, velocity.
static int kernels_per_step(const ts_sim *s) {
    return (s->dims == 3 ? (s->p.stress_pair_3d ? 2 : 3) : 2) + (s->rc.n_chunks > 0 ? 1 : 0);
}

extern "C" {

const char *ts_strerror(int code) {
    switch (code) {
    case TS_OK: return "ok";
    case TS_E_ARG: return "invalid argument";
    case TS_E_CUDA: return "CUDA runtime error";
    case TS_E_NOMEM: return "device memory exhausted";
    case TS_E_NODEV: return "no usable sm_103 device";
    case TS_E_STATE: return "invalid state";
    case TS_E_TIMEOUT: return "wait between thread blocks timed out";
    default: return "unknown error";
    }
}

const char *ts_last_error(void) { return g_last_error.c_str(); }

void ts_destroy(ts_sim *s) {
    if (!s) return;
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(s->device);
    if (s->stream) cudaStreamSynchronize(s->stream);
    if (s->done) cudaEventSynchronize(s->done);
    if (s->graph) cudaGraphExecDestroy(s->graph);
    for (void *d : s->allocs) cudaFree(d);
    if (s->done) cudaEventDestroy(s->done);
    if (s->stream) cudaStreamDestroy(s->stream);
    cudaSetDevice(prev);
    delete s;
}

// Index of the first non-finite value of a float table, or -1.  (Exponent
// bits all set: Inf or NaN; the loop vectorises.)
static int64_t first_non_finite_seq(const uint32_t *u, int64_t n) {
    uint32_t any = 0;
    for (int64_t i = 0; i < n; ++i) any |= ((u[i] & 0x7f800000u) == 0x7f800000u);
    if (!any) return -1;
    for (int64_t i = 0; i < n; ++i)
        if ((u[i] & 0x7f800000u) == 0x7f800000u) return i;
    return -1;
}
static int64_t first_non_finite(const float *a, int64_t n) {
    const uint32_t *u = reinterpret_cast<const uint32_t *>(a);
    constexpr int64_t kChunk = 1 << 20;   // large tables: chunks on parallel threads
    if (n <= kChunk) return first_non_finite_seq(u, n);
    const int chunks = (int)((n + kChunk - 1) / kChunk);
    std::vector<int64_t> first(chunks, -1);
    parallel_rows(chunks, [&](int c) {
        const int64_t i0 = (int64_t)c * kChunk;
        const int64_t i = first_non_finite_seq(u + i0, std::min(kChunk, n - i0));
        if (i >= 0) first[c] = i0 + i;
    });
    for (int64_t i : first)
        if (i >= 0) return i;
    return -1;
}

// Material, coefficients and CPML tables must be finite.  The reference
// does not check them: a NaN there turns the wavefield into NaN, which its
// `norm > threshold` stability test never catches.
static int check_finite(const ts_desc *d, int dims) {
    const int64_t cells = (int64_t)d->nx * d->ny * (dims == 3 ? d->nz : 1);
    struct {
        const char *name;
        const float *a;
        int64_t n;
    } tabs[] = {
        {"rho", d->rho, cells}, {"cp", d->cp, cells}, {"cs", d->cs, cells},
        {"coefs", d->coefs, d->ord},
        {"a_x", d->a_x, d->nx - 2 * (d->ord - 1)}, {"b_x", d->b_x, d->nx - 2 * (d->ord - 1)},
        {"k_x", d->k_x, d->nx - 2 * (d->ord - 1)}, {"a_x_half", d->a_xh, d->nx - 2 * (d->ord - 1)},
        {"b_x_half", d->b_xh, d->nx - 2 * (d->ord - 1)}, {"k_x_half", d->k_xh, d->nx - 2 * (d->ord - 1)},
        {"a_y", d->a_y, d->ny - 2 * (d->ord - 1)}, {"b_y", d->b_y, d->ny - 2 * (d->ord - 1)},
        {"k_y", d->k_y, d->ny - 2 * (d->ord - 1)}, {"a_y_half", d->a_yh, d->ny - 2 * (d->ord - 1)},
        {"b_y_half", d->b_yh, d->ny - 2 * (d->ord - 1)}, {"k_y_half", d->k_yh, d->ny - 2 * (d->ord - 1)},
        {"a_z", dims == 3 ? d->a_z : nullptr, d->nz - 2 * (d->ord - 1)},
        {"b_z", dims == 3 ? d->b_z : nullptr, d->nz - 2 * (d->ord - 1)},
        {"k_z", dims == 3 ? d->k_z : nullptr, d->nz - 2 * (d->ord - 1)},
        {"a_z_half", dims == 3 ? d->a_zh : nullptr, d->nz - 2 * (d->ord - 1)},
        {"b_z_half", dims == 3 ? d->b_zh : nullptr, d->nz - 2 * (d->ord - 1)},
        {"k_z_half", dims == 3 ? d->k_zh : nullptr, d->nz - 2 * (d->ord - 1)},
        {"g_p", d->visco ? d->g_p : nullptr, cells}, {"g_s", d->visco ? d->g_s : nullptr, cells},
    };
    for (const auto &t : tabs) {
        if (!t.a) continue;
        const int64_t i = first_non_finite(t.a, t.n);
        if (i >= 0)
            return fail(TS_E_ARG, std::string("non-finite value in ") + t.name + " at flat index " + std::to_string(i));
    }
    return TS_OK;
}

static int validate(const ts_desc *d) {
    if (!d) return fail(TS_E_ARG, "null descriptor");
    if (d->abi_version != TS_ABI_VERSION) return fail(TS_E_ARG, "abi_version mismatch");
    if (d->family < TS_TAICHI2D || d->family > TS_WGSL3D) return fail(TS_E_ARG, "unknown family");
    if (d->ord < 2 || d->ord > ts::kMaxOrd) return fail(TS_E_ARG, "ord must be in [2, 6]");
    const int dims = d->family == TS_WGSL3D ? 3 : 2;
    const int minn = 2 * d->ord + 1;
    if (d->nx < minn || d->ny < minn || (dims == 3 && d->nz < minn)) return fail(TS_E_ARG, "grid smaller than the stencil");
    if (dims == 2 && d->nz != 1) return fail(TS_E_ARG, "nz must be 1 in 2D");
    if (d->n_steps < 1) return fail(TS_E_ARG, "n_steps must be positive");
    if (!d->coefs || !d->rho || !d->cp || !d->cs) return fail(TS_E_ARG, "missing coefficient or material table");
    if (!d->a_x || !d->b_x || !d->k_x || !d->a_xh || !d->b_xh || !d->k_xh || !d->a_y || !d->b_y || !d->k_y ||
        !d->a_yh || !d->b_yh || !d->k_yh)
        return fail(TS_E_ARG, "missing CPML table");
    if (dims == 3 && (!d->a_z || !d->b_z || !d->k_z || !d->a_zh || !d->b_zh || !d->k_zh))
        return fail(TS_E_ARG, "missing z CPML table");
    if (!(d->dx > 0.f) || !(d->dy > 0.f) || !(d->dt > 0.f) || (dims == 3 && !(d->dz > 0.f)))
        return fail(TS_E_ARG, "grid and time steps must be positive");
    if (d->family == TS_TAICHI2D && d->visco) return fail(TS_E_ARG, "the Taichi family is elastic only");
    if (d->visco) {
        if (d->n_sls < 1 || d->n_sls > ts::kMaxSls) return fail(TS_E_ARG, "n_sls must be in [1, 8]");
        if (!d->g_p && (!d->tau || !d->sum_alpha)) return fail(TS_E_ARG, "missing Zener tables");
        if (d->g_p && (!d->g_s || !d->zc || !d->zh || !d->zm)) return fail(TS_E_ARG, "incomplete per-cell Q tables");
    }
    if (!d->source_term || !d->pos_sources || d->src_rows < 1 || d->src_cols < 1)
        return fail(TS_E_ARG, "missing source term or source map");
    if (d->n_rec < 0 || d->n_rec_pt < 0 || !d->delay_rec) return fail(TS_E_ARG, "bad receiver counts");
    if (d->n_rec > 0 && d->family == TS_TAICHI2D && !d->pos_sensors) return fail(TS_E_ARG, "missing sensor map");
    if (d->n_rec > 0 && d->family != TS_TAICHI2D && (!d->info_rec_pt || !d->offset_sensors))
        return fail(TS_E_ARG, "missing receiver point table");
    return check_finite(d, dims);
}

int ts_create(const ts_desc *d, ts_sim **out) {
    if (!out) return fail(TS_E_ARG, "null output handle");
    *out = nullptr;
    PhaseClock clk;
    int rc = validate(d);
    if (rc) return rc;
    clk.mark("validate");

    int device = 0;
    TS_CUDA(cudaGetDevice(&device));
    int cc_major = 0, cc_minor = 0, n_sms = 0;   // attribute queries: cheaper than the whole property block
    TS_CUDA(cudaDeviceGetAttribute(&cc_major, cudaDevAttrComputeCapabilityMajor, device));
    TS_CUDA(cudaDeviceGetAttribute(&cc_minor, cudaDevAttrComputeCapabilityMinor, device));
    TS_CUDA(cudaDeviceGetAttribute(&n_sms, cudaDevAttrMultiProcessorCount, device));
    if (!(cc_major == 10 && cc_minor == 3)) {
        cudaDeviceProp prop;
        TS_CUDA(cudaGetDeviceProperties(&prop, device));
        return fail(TS_E_NODEV, "device " + std::string(prop.name) + " is sm_" + std::to_string(cc_major) +
                                    std::to_string(cc_minor) + "; this library is built for sm_103a only");
    }

    ts_sim *s = new ts_sim();
    s->device = device;
    s->family = d->family;
    s->dims = d->family == TS_WGSL3D ? 3 : 2;
    s->ord = d->ord;
    s->nx = d->nx;
    s->ny = d->ny;
    s->nz = s->dims == 3 ? d->nz : 1;
    const int last = s->dims == 2 ? s->ny : s->nz;
    s->pitch = round_up(last, 32);
    s->grid_elems = (int64_t)s->nx * (s->dims == 2 ? 1 : s->ny) * s->pitch;
    s->n_rows = d->n_steps;
    s->n_rec = d->n_rec;
    const int nx = s->nx, ny = s->ny, nz = s->nz, ord = s->ord;
    auto bail = [&](int code) {
        ts_destroy(s);
        return code;
    };
    auto href = [&](int x, int y, int z) -> int64_t { return ((int64_t)x * ny + y) * nz + z; };
    auto rho = [&](int x, int y, int z) -> float {
        if (x < 0 || x >= nx || y < 0 || y >= ny || z < 0 || z >= nz) return 0.f;
        return d->rho[href(x, y, z)];
    };
    auto csv = [&](int x, int y, int z) -> float {
        if (x < 0 || x >= nx || y < 0 || y >= ny || z < 0 || z >= nz) return 0.f;
        return d->cs[href(x, y, z)];
    };
    auto cpv = [&](int x, int y, int z) -> float {
        if (x < 0 || x >= nx || y < 0 || y >= ny || z < 0 || z >= nz) return 0.f;
        return d->cp[href(x, y, z)];
    };

    StepParams &p = s->p;
    p.family = s->family;
    // family TS_TAICHI2D: the unbiased arithmetic by default; TS_TAICHI_EXACT=1
    // rounds every operation on its own, bit for bit the float oracle (and the
    // persistent path, which computes that form)
    const char *te = getenv("TS_TAICHI_EXACT");
    p.taichi_exact = te && te[0] == '1';
    // nodes per thread along x (2D; 3D velocity kernel): enough blocks to fill the GPU, as few
    // index/region/bookkeeping instructions per node as that allows
    {
        const int64_t cells = (int64_t)d->nx * d->ny;
        p.tx = s->dims == 3 ? ts::velocity_tx_3d(d->ord) : ts::nodes_per_thread_2d(cells);
        const char *xy = getenv("TS_3D_XY_SWEEP");
        p.xy_sweep_3d = !(xy && xy[0] == '0');
        const char *pair = getenv("TS_3D_STRESS_PAIR");
        p.stress_pair_3d = !(pair && pair[0] == '0');
        // L2 prefetch in the 3D kernels: 2 (default) the state last written
        // two launches back before the wait, 1 after it, 0 none
        // the velocity launch walks the x-chunks backwards, so that each launch
        // starts on the chunks the launch before it wrote last (still in L2)
        const char *sn = getenv("TS_3D_SNAKE");   // "0": forwards
        p.snake_3d = !(sn && sn[0] == '0');
        const char *pf = getenv("TS_3D_PREFETCH");
        p.prefetch_3d = !pf ? 2 : pf[0] == '0' ? 0 : pf[0] == '1' ? 1 : 2;
    }
    p.nx = nx;
    p.ny = ny;
    p.nz = nz;
    p.pitch = s->pitch;
    p.plane = s->dims == 2 ? s->pitch : (int64_t)ny * s->pitch;
    p.grid_elems = s->grid_elems;
    const float steps[3] = {d->dx, d->dy, d->dz};
    for (int a = 0; a < 3; ++a)
        for (int c = 0; c < ts::kMaxOrd; ++c) p.cd[a][c] = c < ord ? d->coefs[c] / steps[a] : 0.f;
    for (int c = 0; c < ts::kMaxOrd; ++c) p.coef[c] = c < ord ? d->coefs[c] : 0.f;
    for (int a = 0; a < 3; ++a) p.od[a] = steps[a] > 0.f ? 1.f / steps[a] : 0.f;
    for (int a = 0; a < 3; ++a) p.dd[a] = steps[a];
    for (int a = 0; a < 3; ++a) p.odl[a] = steps[a] > 0.f ? (float)(1.0 / (double)steps[a] - (double)p.od[a]) : 0.f;
    p.dt = d->dt;

    clk.mark("setup");
    // ---- CPML tables and strips ----
    Axis axes[3];
    axes[0] = make_axis(nx, ord, d->a_x, d->b_x, d->k_x, d->a_xh, d->b_xh, d->k_xh);
    axes[1] = make_axis(ny, ord, d->a_y, d->b_y, d->k_y, d->a_yh, d->b_yh, d->k_yh);
    if (s->dims == 3) axes[2] = make_axis(nz, ord, d->a_z, d->b_z, d->k_z, d->a_zh, d->b_zh, d->k_zh);
    else axes[2] = make_axis(1, ord, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr);
    for (int a = 0; a < 3; ++a) {
        Cpml *f = nullptr, *h = nullptr;
        if ((rc = s->upload(&f, axes[a].full)) || (rc = s->upload(&h, axes[a].half))) return bail(rc);
        p.tab_f[a] = f;
        p.tab_h[a] = h;
        p.strip[a] = axes[a].strip;
    }

    clk.mark("cpml");
    // ---- fields ----
    const int nfields = s->dims == 2 ? 5 : 9;
    const int field_ids2[5] = {TS_VX, TS_VY, TS_SXX, TS_SYY, TS_SXY};
    for (int f = 0; f < nfields; ++f) {
        const int id = s->dims == 2 ? field_ids2[f] : f;
        if ((rc = s->alloc(&s->field[id], s->grid_elems, true))) return bail(rc);
    }
    for (int c = 0; c < 3; ++c) p.v[c] = s->field[TS_VX + c];
    for (int c = 0; c < 6; ++c) p.s[c] = s->field[TS_SXX + c];

    // ---- strip memories ----
    const Strip &sx = p.strip[0], &sy = p.strip[1], &sz = p.strip[2];
    if (s->dims == 2) {
        const int64_t xs = (int64_t)sx.width * s->pitch, ys = (int64_t)nx * sy.width;
        const int64_t sizes[8] = {xs, xs, ys, ys, xs, xs, ys, ys};
        for (int k = 0; k < 8; ++k)
            if ((rc = s->alloc(&p.psi[k], sizes[k], true))) return bail(rc);
    } else {
        const int64_t xs = (int64_t)sx.width * ny * s->pitch, ys = (int64_t)nx * sy.width * s->pitch,
                      zs = (int64_t)nx * ny * sz.width;
        // stress: 0 x, 1 y, 2 z, 3 x, 4 y, 5 x, 6 z, 7 y, 8 z; velocity: 9 x, 10 y, 11 z, 12 x, 13 y, 14 z, 15 x, 16 y, 17 z
        const char axis_of[18] = {'x', 'y', 'z', 'x', 'y', 'x', 'z', 'y', 'z',
                                  'x', 'y', 'z', 'x', 'y', 'z', 'x', 'y', 'z'};
        for (int k = 0; k < 18; ++k) {
            const int64_t n = axis_of[k] == 'x' ? xs : axis_of[k] == 'y' ? ys : zs;
            if ((rc = s->alloc(&p.psi[k], n, true))) return bail(rc);
        }
    }

    clk.mark("fields");
    // ---- per-node coefficients (host, reference averaging; raw: the kernels
    // multiply by dt and divide by rho as the reference does) ----
    const size_t ng = (size_t)s->grid_elems;
    hvec lam = filled(ng, 0.f), mu = filled(ng, 0.f), dtr0 = filled(ng, 0.f), dtr1 = filled(ng, 0.f);
    hvec mus[3];
    const int n_shear = s->dims == 2 ? 1 : 3;
    for (int k = 0; k < n_shear; ++k) mus[k] = filled(ng, 0.f);
    if (s->dims == 2) {
        // normal node x-averaged (mu zero where either cs is zero), shear
        // node y-averaged, vy node 4-point averaged (ts_prep.h)
        parallel_rows(nx, [&](int x) {
            for (int y = 0; y < ny; ++y) {
                const int64_t i = s->at(x, y);
                const ts::Coef2D c = ts::coef_2d(d, x, y);
                // raw moduli and densities: the kernels multiply by dt and
                // divide by rho as the reference does
                lam[i] = c.lam_raw;
                mu[i] = c.mu_raw;
                mus[0][i] = c.mus_raw;
                dtr0[i] = c.rho_vx;
                dtr1[i] = c.rho_vy;
            }
        });
    } else {
        // one expression for every node; `at(a, b, c)` reads (rho, cs, cp) at
        // (x + a, y + b, z + c), without bounds tests away from the far faces
        auto node = [&](int64_t i, const auto &rho_at, const auto &cs_at, float cp) {
            const float r = rho_at(0, 0, 0), cs = cs_at(0, 0, 0);
            lam[i] = r * (cp * cp - 2.f * cs * cs);   // raw: the kernels multiply by dt
            mu[i] = r * (cs * cs);
            const float rxy = 0.25f * (rho_at(1, 0, 0) + rho_at(0, 0, 0) + rho_at(0, 1, 0) + rho_at(1, 1, 0));
            const float cxy = 0.25f * (cs_at(1, 0, 0) + cs_at(0, 0, 0) + cs_at(0, 1, 0) + cs_at(1, 1, 0));
            const float rxz = 0.25f * (rho_at(1, 0, 0) + rho_at(0, 0, 0) + rho_at(0, 0, 1) + rho_at(1, 0, 1));
            const float cxz = 0.25f * (cs_at(1, 0, 0) + cs_at(0, 0, 0) + cs_at(0, 0, 1) + cs_at(1, 0, 1));
            const float ryz = 0.25f * (rho_at(0, 1, 0) + rho_at(0, 0, 0) + rho_at(0, 0, 1) + rho_at(0, 1, 1));
            const float cyz = 0.25f * (cs_at(0, 1, 0) + cs_at(0, 0, 0) + cs_at(0, 0, 1) + cs_at(0, 1, 1));
            mus[0][i] = rxy * (cxy * cxy);
            mus[1][i] = rxz * (cxz * cxz);
            mus[2][i] = ryz * (cyz * cyz);
            dtr0[i] = 0.5f * (rho_at(1, 0, 0) + r);   // raw: the kernels divide by rho
            dtr1[i] = 0.5f * (rho_at(0, 1, 0) + r);
        };
        const int64_t SX = (int64_t)ny * nz, SY = nz;
        parallel_rows(nx, [&](int x) {
            for (int y = 0; y < ny; ++y)
                for (int z = 0; z < nz; ++z) {
                    const int64_t i = s->at(x, y, z), h = href(x, y, z);
                    if (x + 1 < nx && y + 1 < ny && z + 1 < nz) {
                        const float *R = d->rho + h, *C = d->cs + h;
                        node(i, [&](int a, int b, int c) { return R[a * SX + b * SY + c]; },
                             [&](int a, int b, int c) { return C[a * SX + b * SY + c]; }, d->cp[h]);
                    } else {
                        node(i, [&](int a, int b, int c) { return rho(x + a, y + b, z + c); },
                             [&](int a, int b, int c) { return csv(x + a, y + b, z + c); }, cpv(x, y, z));
                    }
                }
        });
    }
    clk.mark("coefficients");
    // ---- attenuation ----
    s->zen_mode = !d->visco ? 0 : (d->g_p ? 2 : 1);
    hvec gp, gs;
    if (d->visco) {
        const int L = d->n_sls;
        p.zen = ts::zener_constants(d);
        const int nmem = s->dims == 2 ? 3 : 6;
        for (int m = 0; m < nmem; ++m)
            if ((rc = s->alloc(&p.r[m], s->grid_elems * L, true))) return bail(rc);
        if (s->zen_mode == 2) {
            gp = filled(ng, 0.f);
            gs = filled(ng, 0.f);
            parallel_rows(nx, [&](int x) {
                for (int y = 0; y < ny; ++y)
                    for (int z = 0; z < nz; ++z) {
                        gp[s->at(x, y, z)] = d->g_p[href(x, y, z)];
                        gs[s->at(x, y, z)] = d->g_s[href(x, y, z)];
                    }
            });
        }
    }

    clk.mark("attenuation");
    // ---- coefficients to the device: a palette (3D, 32-bit offsets) or arrays ----
    float *dev = nullptr;
    bool palette = false;
    const char *pal_env = getenv("TS_3D_COEF_PALETTE");   // "0": arrays (tests cover both paths)
    const char *pal2_env = getenv("TS_2D_COEF_PALETTE");  // "0": arrays
    const bool pal3 = s->dims == 3 && s->grid_elems * (int64_t)std::max(1, p.zen.n) < ((int64_t)1 << 31) &&
                      !(pal_env && pal_env[0] == '0');
    const char *pers_env = getenv("TS_2D_PERSISTENT");     // the persistent kernel reads the arrays
    const bool pal2 = s->dims == 2 && s->family == TS_WGSL2D && ord == 2 && !(pal2_env && pal2_env[0] == '0') &&
                      !(pers_env && pers_env[0] == '1');
    if (pal3 || pal2) {
        const hvec ones = filled(gp.empty() ? ng : 0, 1.f);
        const hvec zeros = filled(pal2 ? ng : 0, 0.f);
        const hvec *cols[7] = {&lam, &mu, gp.empty() ? &ones : &gp, gs.empty() ? &ones : &gs,
                                             &mus[0], pal2 ? &zeros : &mus[1], pal2 ? &zeros : &mus[2]};
        std::vector<uint16_t> idx;
        std::vector<ts::Pal3> table;
        if (build_palette_3d(cols, nx, idx, table)) {
            uint16_t *didx = nullptr;
            ts::Pal3 *dtab = nullptr;
            if ((rc = s->upload(&didx, idx)) || (rc = s->upload(&dtab, table))) return bail(rc);
            p.pal_idx = didx;
            p.pal = dtab;
            palette = true;
        }
    }
    if (s->dims == 2) {   // rho itself: the 2D kernels divide by it
        if ((rc = s->upload(&dev, dtr0))) return bail(rc);
        p.dtr[0] = dev;
        if ((rc = s->upload(&dev, dtr1))) return bail(rc);
        p.dtr[1] = dev;
    } else {   // dt / rho as (hi, lo) pairs
        for (int c = 0; c < 2; ++c) {
            const hvec &rh = c == 0 ? dtr0 : dtr1;
            std::vector<float2> w(rh.size());
            const size_t per = (rh.size() + nx - 1) / nx;
            parallel_rows(nx, [&](int x) {
                for (size_t i = x * per; i < std::min(rh.size(), (x + 1) * per); ++i) w[i] = dt_over_rho(d->dt, rh[i]);
            });
            float2 *dw = nullptr;
            if ((rc = s->upload(&dw, w))) return bail(rc);
            p.dtw[c] = dw;
        }
        p.dtw[2] = p.dtw[1];   // vz uses the vy-node density (wgsl3d:1748)
    }
    if (!palette) {
        if ((rc = s->upload(&dev, lam))) return bail(rc);
        p.lam_dt = dev;
        if ((rc = s->upload(&dev, mu))) return bail(rc);
        p.mu_dt = dev;
        for (int k = 0; k < n_shear; ++k) {
            if ((rc = s->upload(&dev, mus[k]))) return bail(rc);
            p.mus_dt[k] = dev;
        }
        if (s->zen_mode == 2) {
            if ((rc = s->upload(&dev, gp))) return bail(rc);
            p.g_p = dev;
            if ((rc = s->upload(&dev, gs))) return bail(rc);
            p.g_s = dev;
        }
    }

    clk.mark("coef upload");
    // ---- launch geometry ----
    s->n_blocks = s->dims == 2 ? ts::blocks_2d(p) : ts::blocks_3d(p);
    auto block_of = [&](int x, int y, int z) -> int {
        return s->dims == 2 ? ts::block_of_2d(p, x, y) : ts::block_of_3d(p, x, y, z);
    };

    // host copies the persistent path rebuilds its own lists from
    std::vector<Source> src_list_h;
    std::vector<int> rec_start_h;
    std::vector<int64_t> rec_cells_h;

    // ---- sources ----
    {
        s->src_rows = d->src_rows;
        s->src_cols_in = d->src_cols;
        s->n_src_el = d->n_src_el;
        struct Cand {
            int blk;
            Source s;
        };
        std::vector<Cand> cands;
        std::map<int, int> col_of;
        // the nodes whose map entry is not -1, found in parallel, then taken
        // in the reference's scan order
        std::vector<std::vector<int2>> marked(nx);
        parallel_rows(nx, [&](int x) {
            for (int y = 0; y < ny; ++y)
                for (int z = 0; z < nz; ++z)
                    if (d->pos_sources[href(x, y, z)] != -1) marked[x].push_back(make_int2(y, z));
        });
        for (int x = 0; x < nx; ++x)
            for (const int2 yz : marked[x]) {
                const int y = yz.x, z = yz.y;
                const int idx = d->pos_sources[href(x, y, z)];
                float r;
                if (s->family == TS_TAICHI2D) {
                    const bool in_vy = x >= ord - 1 && x < nx - ord && y >= ord - 1 && y < ny - ord;
                    if (!in_vy || idx < 0 || idx >= d->src_cols) continue;
                    r = 0.25f * (rho(x, y + 1, 0) + rho(x, y, 0) + rho(x + 1, y + 1, 0) + rho(x + 1, y, 0));
                } else if (s->dims == 2) {
                    r = 0.25f * (rho(x, y, 0) + rho(x + 1, y, 0) + rho(x + 1, y + 1, 0) + rho(x, y + 1, 0));
                } else {
                    r = 0.5f * (rho(x, y + 1, z) + rho(x, y, z));
                }
                if (!(r > 0.f)) continue;
                const float scale = r;   // the kernels divide by rho
                if (!col_of.count(idx)) {
                    const int c = (int)col_of.size();
                    col_of[idx] = c;
                    s->src_col_idx.push_back(idx);
                }
                cands.push_back({block_of(x, y, z), Source{s->at(x, y, z), col_of[idx], scale}});
            }
        std::stable_sort(cands.begin(), cands.end(), [](const Cand &a, const Cand &b) { return a.blk < b.blk; });
        std::vector<Source> &list = src_list_h;
        std::vector<int> start(s->n_blocks + 1, 0);
        for (const Cand &c : cands) {
            list.push_back(c.s);
            start[c.blk + 1]++;
        }
        for (int b = 0; b < s->n_blocks; ++b) start[b + 1] += start[b];
        Source *dsrc = nullptr;
        int *dstart = nullptr;
        if ((rc = s->upload(&dsrc, list)) || (rc = s->upload(&dstart, start))) return bail(rc);
        p.src = dsrc;
        p.src_block_start = dstart;
        p.src_rows = d->src_rows;
        p.src_ncol = std::max<int>(1, (int)s->src_col_idx.size());
        if ((rc = s->alloc(&s->src_tab, (size_t)p.src_rows * p.src_ncol, false))) return bail(rc);
        p.src_tab = s->src_tab;
        if ((rc = ts_set_sources(s, d->source_term))) return bail(rc);
    }

    clk.mark("sources");
    // ---- receivers ----
    {
        std::vector<int> start(1, 0), first(d->n_rec, 0);
        std::vector<int64_t> cells;
        if (s->family == TS_TAICHI2D) {
            std::vector<std::vector<int64_t>> per(d->n_rec);
            for (int x = ord - 1; x < nx - ord; ++x)
                for (int y = ord; y < ny - ord + 1; ++y) {
                    const int sn = d->pos_sensors[href(x, y, 0)];
                    if (sn >= 0 && sn < d->n_rec) per[sn].push_back(s->at(x, y));
                }
            for (int r = 0; r < d->n_rec; ++r) {
                cells.insert(cells.end(), per[r].begin(), per[r].end());
                start.push_back((int)cells.size());
                first[r] = d->delay_rec[r] - 1;  // 1-based it >= delay
            }
        } else {
            const int cols = 1 + s->dims;  // [ix, iy(, iz), receiver]
            const int rec_groups = ts::receiver_groups(d, cols);
            for (int r = 0; r < d->n_rec; ++r) {
                for (int pt = ts::receiver_first_point(d, r, rec_groups); pt >= 0 && pt < d->n_rec_pt && d->info_rec_pt[pt * cols + cols - 1] == r;
                     ++pt) {
                    const int *q = d->info_rec_pt + pt * cols;
                    const int x = q[0], y = q[1], z = s->dims == 3 ? q[2] : 0;
                    if (x < 0 || x >= nx || y < 0 || y >= ny || z < 0 || z >= nz) continue;  // reads as 0
                    cells.push_back(s->at(x, y, z));
                }
                start.push_back((int)cells.size());
                first[r] = d->delay_rec[r];
            }
        }
        int *ds = nullptr, *df = nullptr;
        int64_t *dc = nullptr;
        if ((rc = s->upload(&ds, start)) || (rc = s->upload(&df, first)) || (rc = s->upload(&dc, cells))) return bail(rc);
        rec_start_h = start;
        rec_cells_h = cells;
        p.n_rec = d->n_rec;
        p.rec_start = ds;
        p.rec_first_step = df;
        p.rec_cell = dc;
        if ((rc = s->alloc(&s->traces, (size_t)s->n_rows * std::max(1, d->n_rec), true))) return bail(rc);
        p.traces = s->traces;
    }

    clk.mark("receivers");
    // ---- stability bookkeeping ----
    p.v2_threshold = s->family == TS_TAICHI2D ? 1.0e38f : FLT_MAX;
    if ((rc = s->alloc(&s->block_max, s->n_blocks, true)) || (rc = s->alloc(&s->first_bad, 1, false)) ||
        (rc = s->alloc(&s->step_base, 1, false)))
        return bail(rc);
    p.block_max = s->block_max;
    p.first_bad = s->first_bad;
    p.step_base = s->step_base;

    // ---- persistent path (opt-in, TS_2D_PERSISTENT=1): 2D elastic order-2
    // models whose row slabs fit on chip.  Measured slower than the stepped
    // path on GB300 (the per-step compute of a slab, half of it recomputed
    // halo rows, runs at 16 warps per SM), so it is not the default. ----
    if (s->dims == 2) {
        const char *env = getenv("TS_2D_PERSISTENT");
        int rows = 0, blocks = 0, threads = 0;
        size_t smem = 0;
        if (env && env[0] == '1' &&
            ts::persist_2d_plan(s->family, ord, s->zen_mode, nx, ny, p.strip[1].width, n_sms,
                                &rows, &blocks, &threads, &smem)) {
            ts::PersistArgs &a = s->pa;
            constexpr int NH = 3;   // 2 ORD - 1 edge rows per side
            const int64_t n_pts = (int64_t)rec_cells_h.size();
            if ((rc = s->alloc(&a.mail, (size_t)blocks * 2 * 2 * 2 * NH * threads, false)) ||
                (rc = s->alloc(&a.flags, blocks, true)) || (rc = s->alloc(&a.err, 4, true)) ||
                (rc = s->alloc(&a.samples, (size_t)s->n_rows * std::max<int64_t>(n_pts, 1), false)))
                return bail(rc);
            // receiver points and source nodes, each by the block whose slab holds its row
            std::vector<std::vector<int4>> by_pt(blocks), by_src(blocks);
            for (int64_t q = 0; q < n_pts; ++q) {
                const int x = (int)(rec_cells_h[q] / s->pitch), y = (int)(rec_cells_h[q] % s->pitch);
                by_pt[x / rows].push_back(make_int4(x % rows, y, (int)q, 0));
            }
            for (const Source &src : src_list_h) {
                const int x = (int)(src.cell / s->pitch), y = (int)(src.cell % s->pitch);
                int bits;
                std::memcpy(&bits, &src.scale, 4);
                by_src[x / rows].push_back(make_int4(x % rows, y, src.col, bits));
            }
            std::vector<int4> pts, srcs;
            std::vector<int> pts_start(1, 0), src_start(1, 0);
            for (int b = 0; b < blocks; ++b) {
                pts.insert(pts.end(), by_pt[b].begin(), by_pt[b].end());
                srcs.insert(srcs.end(), by_src[b].begin(), by_src[b].end());
                pts_start.push_back((int)pts.size());
                src_start.push_back((int)srcs.size());
            }
            int4 *dpts = nullptr, *dsrcs = nullptr;
            int *dps = nullptr, *dss = nullptr;
            if ((rc = s->upload(&dpts, pts)) || (rc = s->upload(&dps, pts_start)) || (rc = s->upload(&dsrcs, srcs)) ||
                (rc = s->upload(&dss, src_start)))
                return bail(rc);
            a.pts = dpts;
            a.pts_start = dps;
            a.srcs = dsrcs;
            a.src_start = dss;
            a.n_pts = (int)n_pts;
            a.n_blocks = s->n_blocks;
            a.wait_ns = 1000000000LL;   // 1 s
            if (const char *w = getenv("TS_PERSIST_WAIT_NS")) a.wait_ns = std::max(1000LL, atoll(w));
            a.stall_block = -1;
            if (const char *b = getenv("TS_PERSIST_STALL_BLOCK")) a.stall_block = atoi(b);
            s->persist = 1;
            s->p_rows = rows;
            s->p_blocks = blocks;
            s->p_threads = threads;
            s->p_smem = smem;
        }
    }

    // ---- receivers with many points: summed in chunks after each step (stepped path) ----
    if (!s->persist && d->n_rec > 0) {
        const char *force = getenv("TS_RECEIVER_CHUNKS");          // 1: every receiver chunked
        const char *cp = getenv("TS_RECEIVER_CHUNK_POINTS");      // chunk size
        const bool all = force && force[0] == '1';
        const int per = cp ? std::max(1, atoi(cp)) : ts::kChunkPoints;
        std::vector<unsigned char> flag(d->n_rec, 0);
        std::vector<int2> chunks;
        std::vector<int> recv, rchunk(1, 0);
        for (int r = 0; r < d->n_rec; ++r) {
            const int a = rec_start_h[r], b = rec_start_h[r + 1];
            if (!(all || b - a > ts::kChunkedMinPoints)) continue;
            flag[r] = 1;
            recv.push_back(r);
            for (int q = a; q < b; q += per) chunks.push_back(make_int2(q, std::min(b, q + per)));
            rchunk.push_back((int)chunks.size());
        }
        if (!chunks.empty()) {
            unsigned char *dflag = nullptr;
            int2 *dch = nullptr;
            int *drecv = nullptr, *drch = nullptr;
            if ((rc = s->upload(&dflag, flag)) || (rc = s->upload(&dch, chunks)) || (rc = s->upload(&drecv, recv)) ||
                (rc = s->upload(&drch, rchunk)) || (rc = s->alloc(&s->rc.partial, chunks.size(), false)) ||
                (rc = s->alloc(&s->rc.counter, 1, true)))
                return bail(rc);
            p.rec_chunked = dflag;
            s->rc.n_chunks = (int)chunks.size();
            s->rc.n_chunked = (int)recv.size();
            s->rc.chunk = dch;
            s->rc.receiver = drecv;
            s->rc.rchunk = drch;
            s->rc.cell = p.rec_cell;
        }
    }

    clk.mark("paths");
    cudaError_t e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) return bail(cuda_fail(e, "cudaStreamCreate"));
    e = cudaEventCreateWithFlags(&s->done, cudaEventDisableTiming);
    if (e != cudaSuccess) return bail(cuda_fail(e, "cudaEventCreate"));
    if ((rc = ts_reset(s))) return bail(rc);
    clk.mark("reset");
    *out = s;
    return TS_OK;
}

int ts_set_sources(ts_sim *s, const float *source_term) {
    if (!s || !source_term) return fail(TS_E_ARG, "null argument");
    const int rows = s->src_rows, ncol = s->p.src_ncol;
    std::vector<float> tab((size_t)rows * ncol, 0.f);
    for (int c = 0; c < (int)s->src_col_idx.size(); ++c) {
        const int idx = s->src_col_idx[c];
        for (int k = 0; k < rows; ++k) {
            float v = 0.f;
            if (s->family == TS_TAICHI2D) {
                v = source_term[(int64_t)k * s->src_cols_in + idx];
            } else if (idx >= 0 && idx < s->n_src_el && k < s->n_rows) {
                const int64_t flat = (int64_t)k * s->n_src_el + idx;
                if (flat < (int64_t)rows * s->src_cols_in) v = source_term[flat];
            }
            tab[(size_t)k * ncol + c] = v;
        }
    }
    if (s->done) TS_CUDA(cudaEventSynchronize(s->done));
    TS_CUDA(cudaMemcpy(s->src_tab, tab.data(), tab.size() * sizeof(float), cudaMemcpyHostToDevice));
    s->h2d_bytes += (int64_t)(tab.size() * sizeof(float));
    return TS_OK;
}

int ts_reset_async(ts_sim *s, void *stream) {
    if (!s) return fail(TS_E_ARG, "null handle");
    TS_CUDA(cudaSetDevice(s->device));
    cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : s->stream;
    for (size_t k = 0; k < s->state_ptrs.size(); ++k)
        TS_CUDA(cudaMemsetAsync(s->state_ptrs[k], 0, s->state_bytes[k], st));
    ts::launch_reset_scalars(s->first_bad, s->step_base, st);
    s->launches += 1;
    TS_CUDA(cudaGetLastError());
    TS_CUDA(cudaEventRecord(s->done, st));
    s->steps_done = 0;
    return TS_OK;
}

int ts_reset(ts_sim *s) {
    int rc = ts_reset_async(s, nullptr);
    if (rc) return rc;
    TS_CUDA(cudaStreamSynchronize(s->stream));
    return TS_OK;
}

int ts_profile_steps(ts_sim *s, int32_t n_steps, void *stream, float *ms_per_kernel) {
    if (!s || !ms_per_kernel) return fail(TS_E_ARG, "null argument");
    if (n_steps < 1 || s->steps_done + (int64_t)n_steps > s->n_rows)
        return fail(TS_E_ARG, "steps beyond the source/trace length");
    TS_CUDA(cudaSetDevice(s->device));
    cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : s->stream;
    if (s->persist) {   // one launch for all steps: [0] its time per step, [1] the receiver sums' per step
        cudaEvent_t e0, e1, e2;
        TS_CUDA(cudaEventCreate(&e0));
        TS_CUDA(cudaEventCreate(&e1));
        TS_CUDA(cudaEventCreate(&e2));
        s->pa.p = s->p;
        s->pa.n_steps = n_steps;
        const int n_rec = s->pa.p.n_rec;
        s->pa.p.n_rec = 0;   // the kernel alone, then the receiver sums
        TS_CUDA(cudaEventRecord(e0, st));
        cudaError_t e = ts::launch_persist_2d(s->pa, s->family, s->p_rows, s->p_blocks, s->p_threads, s->p_smem, st);
        s->pa.p.n_rec = n_rec;
        if (e != cudaSuccess) return cuda_fail(e, "persistent step launch");
        TS_CUDA(cudaEventRecord(e1, st));
        if (n_rec > 0) {
            // receiver sums of the same steps: the kernel's samples, summed by the same launch helper
            ts::PersistArgs r = s->pa;
            r.n_steps = 0;
            TS_CUDA(ts::launch_persist_2d_receivers(r, n_steps, st));
        }
        TS_CUDA(cudaEventRecord(e2, st));
        ts::launch_advance(s->step_base, n_steps, st);
        s->launches += 2 + (n_rec > 0 ? 1 : 0);
        TS_CUDA(cudaEventSynchronize(e2));
        float a = 0.f, b = 0.f;
        TS_CUDA(cudaEventElapsedTime(&a, e0, e1));
        TS_CUDA(cudaEventElapsedTime(&b, e1, e2));
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        cudaEventDestroy(e2);
        ms_per_kernel[0] = a / n_steps;
        ms_per_kernel[1] = b / n_steps;
        TS_CUDA(cudaEventRecord(s->done, st));
        s->steps_done += n_steps;
        return TS_OK;
    }
    std::vector<cudaEvent_t> ev(2 * n_steps + 1);
    for (auto &e : ev) TS_CUDA(cudaEventCreate(&e));
    TS_CUDA(cudaEventRecord(ev[0], st));
    for (int j = 0; j < n_steps; ++j) {
        for (int part = 0; part < 2; ++part) {
            if (s->dims == 2) ts::launch_step_2d(s->p, s->ord, s->zen_mode, j, st, 1 << part);
            else ts::launch_step_3d(s->p, s->ord, s->zen_mode, j, st, 1 << part);
            if (part == 1) ts::launch_receiver_chunks(s->p, s->rc, j, st);   // with the velocity update
            TS_CUDA(cudaEventRecord(ev[2 * j + part + 1], st));
        }
    }
    ts::launch_advance(s->step_base, n_steps, st);
    s->launches += (int64_t)kernels_per_step(s) * n_steps + 1;
    TS_CUDA(cudaGetLastError());
    TS_CUDA(cudaEventSynchronize(ev.back()));
    double tot[2] = {0.0, 0.0};
    for (int j = 0; j < n_steps; ++j)
        for (int part = 0; part < 2; ++part) {
            float ms = 0.f;
            TS_CUDA(cudaEventElapsedTime(&ms, ev[2 * j + part], ev[2 * j + part + 1]));
            tot[part] += ms;
        }
    for (auto &e : ev) cudaEventDestroy(e);
    ms_per_kernel[0] = (float)(tot[0] / n_steps);
    ms_per_kernel[1] = (float)(tot[1] / n_steps);
    TS_CUDA(cudaEventRecord(s->done, st));
    s->steps_done += n_steps;
    return TS_OK;
}

int ts_transfer_bytes(const ts_sim *s, int64_t *h2d, int64_t *d2h) {
    if (!s) return fail(TS_E_ARG, "null handle");
    if (h2d) *h2d = s->h2d_bytes;
    if (d2h) *d2h = s->d2h_bytes;
    return TS_OK;
}

int ts_launch_count(const ts_sim *s, int64_t *launches) {
    if (!s || !launches) return fail(TS_E_ARG, "null argument");
    *launches = s->launches;
    return TS_OK;
}

int ts_run(ts_sim *s, int32_t n_steps, void *stream) {
    if (!s) return fail(TS_E_ARG, "null handle");
    if (n_steps < 0 || s->steps_done + (int64_t)n_steps > s->n_rows)
        return fail(TS_E_ARG, "steps beyond the source/trace length");
    TS_CUDA(cudaSetDevice(s->device));
    cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : s->stream;
    if (s->persist) {   // every step of this call in one cooperative launch
        if (n_steps > 0) {
            s->pa.p = s->p;
            s->pa.n_steps = n_steps;
            cudaError_t e = ts::launch_persist_2d(s->pa, s->family, s->p_rows, s->p_blocks, s->p_threads, s->p_smem, st);
            if (e != cudaSuccess) return cuda_fail(e, "persistent step launch");
            ts::launch_advance(s->step_base, n_steps, st);
            s->launches += 2 + (s->n_rec > 0 ? 1 : 0);
        }
        TS_CUDA(cudaGetLastError());
        TS_CUDA(cudaEventRecord(s->done, st));
        s->steps_done += n_steps;
        return TS_OK;
    }
    auto launch_steps = [&](int count, cudaStream_t where) {
        for (int j = 0; j < count; ++j) {
            if (s->dims == 2) ts::launch_step_2d(s->p, s->ord, s->zen_mode, j, where);
            else ts::launch_step_3d(s->p, s->ord, s->zen_mode, j, where);
            ts::launch_receiver_chunks(s->p, s->rc, j, where);
        }
        ts::launch_advance(s->step_base, count, where);
    };
    if (!s->graph && n_steps >= kGraphSteps) {
        cudaGraph_t g = nullptr;
        TS_CUDA(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
        launch_steps(kGraphSteps, s->stream);
        TS_CUDA(cudaStreamEndCapture(s->stream, &g));
        cudaError_t e = cudaGraphInstantiate(&s->graph, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
    }
    int left = n_steps;
    while (left >= kGraphSteps && s->graph) {
        TS_CUDA(cudaGraphLaunch(s->graph, st));
        s->launches += kernels_per_step(s) * kGraphSteps + 1;
        left -= kGraphSteps;
    }
    if (left > 0) {
        launch_steps(left, st);
        s->launches += kernels_per_step(s) * left + 1;
    }
    TS_CUDA(cudaGetLastError());
    TS_CUDA(cudaEventRecord(s->done, st));
    s->steps_done += n_steps;
    return TS_OK;
}

int ts_status(ts_sim *s, int32_t *steps_done, float *max_v2, int32_t *first_unstable) {
    if (!s) return fail(TS_E_ARG, "null handle");
    TS_CUDA(cudaSetDevice(s->device));
    TS_CUDA(cudaEventSynchronize(s->done));
    if (steps_done) *steps_done = s->steps_done;
    if (s->persist) {
        int err[4] = {0, 0, 0, 0};
        TS_CUDA(cudaMemcpy(err, s->pa.err, sizeof err, cudaMemcpyDeviceToHost));
        if (err[0])
            return fail(TS_E_TIMEOUT, "persistent step kernel: block " + std::to_string(err[2]) +
                                          " gave up waiting for a neighbouring block at step " + std::to_string(err[1]) +
                                          "; the wavefield is invalid until ts_reset");
    }
    if (max_v2) {
        std::vector<unsigned> bm(s->n_blocks);
        TS_CUDA(cudaMemcpy(bm.data(), s->block_max, bm.size() * sizeof(unsigned), cudaMemcpyDeviceToHost));
        unsigned m = 0;
        for (unsigned v : bm) m = std::max(m, v);
        float f;
        std::memcpy(&f, &m, sizeof(f));
        *max_v2 = f;
    }
    if (first_unstable) {
        int fb = 0;
        TS_CUDA(cudaMemcpy(&fb, s->first_bad, sizeof(int), cudaMemcpyDeviceToHost));
        *first_unstable = fb == 0x7fffffff ? -1 : fb;
    }
    return TS_OK;
}

int ts_read(ts_sim *s, int32_t what, void *dst, size_t bytes) {
    if (!s || !dst) return fail(TS_E_ARG, "null argument");
    TS_CUDA(cudaSetDevice(s->device));
    TS_CUDA(cudaEventSynchronize(s->done));
    if (what == TS_TRACES) {
        const size_t need = (size_t)s->n_rows * s->n_rec * sizeof(float);
        if (bytes < need) return fail(TS_E_ARG, "destination too small for the traces");
        if (need) TS_CUDA(stage_d2h(dst, s->traces, (size_t)s->n_rec * sizeof(float), (size_t)s->n_rec * sizeof(float),
                                    (size_t)s->n_rows, s->stream));
        s->d2h_bytes += (int64_t)need;
        return TS_OK;
    }
    if (what < TS_VX || what > TS_SYZ || !s->field[what]) return fail(TS_E_ARG, "no such field");
    const int last = s->dims == 2 ? s->ny : s->nz;
    const size_t rows = (size_t)s->nx * (s->dims == 2 ? 1 : s->ny);
    const size_t need = rows * last * sizeof(float);
    if (bytes < need) return fail(TS_E_ARG, "destination too small for the field");
    TS_CUDA(stage_d2h(dst, s->field[what], last * sizeof(float), s->pitch * sizeof(float), rows, s->stream));
    s->d2h_bytes += (int64_t)need;
    return TS_OK;
}

int ts_device_buffer(ts_sim *s, int32_t what, void **dev_ptr, size_t *pitch_bytes) {
    if (!s || !dev_ptr) return fail(TS_E_ARG, "null argument");
    if (what == TS_TRACES) {
        *dev_ptr = s->traces;
        if (pitch_bytes) *pitch_bytes = (size_t)s->n_rec * sizeof(float);
        return TS_OK;
    }
    if (what < TS_VX || what > TS_SYZ || !s->field[what]) return fail(TS_E_ARG, "no such field");
    *dev_ptr = s->field[what];
    if (pitch_bytes) *pitch_bytes = (size_t)s->pitch * sizeof(float);
    return TS_OK;
}

int ts_copy_field(ts_sim *s, int32_t what, void *dst, size_t dst_pitch, void *stream) {
    if (!s || !dst) return fail(TS_E_ARG, "null argument");
    if (what < TS_VX || what > TS_SYZ || !s->field[what]) return fail(TS_E_ARG, "no such field");
    TS_CUDA(cudaSetDevice(s->device));
    cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : s->stream;
    const int last = s->dims == 2 ? s->ny : s->nz;
    const size_t rows = (size_t)s->nx * (s->dims == 2 ? 1 : s->ny);
    const size_t width = (size_t)last * sizeof(float);
    if (dst_pitch == 0) dst_pitch = width;
    if (dst_pitch < width) return fail(TS_E_ARG, "dst_pitch smaller than a row");
    TS_CUDA(cudaMemcpy2DAsync(dst, dst_pitch, s->field[what], (size_t)s->pitch * sizeof(float), width, rows,
                              cudaMemcpyDefault, st));
    return TS_OK;
}

int ts_step_path(const ts_sim *s, int32_t *path) {
    if (!s || !path) return fail(TS_E_ARG, "null argument");
    *path = s->persist ? TS_PATH_PERSISTENT : TS_PATH_STEPPED;
    return TS_OK;
}

int ts_launches_per_step(const ts_sim *s, int32_t *launches) {
    if (!s || !launches) return fail(TS_E_ARG, "null argument");
    *launches = kernels_per_step(s);
    return TS_OK;
}

}  // extern "C"
