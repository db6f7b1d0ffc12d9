// liblgpu_gb300: errors, device and memory services, scratch contexts, state
// preparation, and the BLAS-1 style kernels (copy, axpy, scale, dot).
#include <atomic>
#include <cstdlib>
#include <mutex>

#include "lgpu_internal.cuh"
#include "lgpu_reduce.cuh"

namespace lgpu {

static thread_local std::string g_last_error;

void set_error(const std::string &msg) { g_last_error = msg; }

lgpu_status_t fail(lgpu_status_t st, const std::string &msg) {
    set_error(msg);
    return st;
}

lgpu_status_t cuda_fail(cudaError_t e, const char *what) {
    std::string msg = std::string("CUDA error in ") + what + ": " + cudaGetErrorName(e) + " (" +
                      cudaGetErrorString(e) + ")";
    if (e == cudaErrorMemoryAllocation) return fail(LGPU_ERR_OOM, msg);
    return fail(LGPU_ERR_CUDA, msg);
}

static std::atomic<unsigned> g_reset_epoch{0};

unsigned reset_epoch() { return g_reset_epoch.load(std::memory_order_acquire); }

// Drops the host-side caches that refer to device `dev`'s context (pooled
// contexts, the static scratch address); defined with those caches below.
void forget_device_state(int dev);

static std::atomic<int> g_f64_mode{-1};

int f64_mode() {
    int m = g_f64_mode.load(std::memory_order_relaxed);
    if (m < 0) {
        const char *e = std::getenv("LGPU_F64_EMUL");
        m = (e && e[0] == '0') ? 0 : 1;
        g_f64_mode.store(m, std::memory_order_relaxed);
    }
    return m;
}

static std::atomic<int> g_bulk_mode{-1};

int bulk_enabled() {
    int m = g_bulk_mode.load(std::memory_order_relaxed);
    if (m < 0) {
        const char *e = std::getenv("LGPU_BULK");
        m = (e && e[0] == '0') ? 0 : 1;
        g_bulk_mode.store(m, std::memory_order_relaxed);
    }
    return m;
}

static std::atomic<int> g_fused_df_mode{-1};

int fused_df_enabled() {
    int m = g_fused_df_mode.load(std::memory_order_relaxed);
    if (m < 0) {
        const char *e = std::getenv("LGPU_FUSED_DF");
        m = (e && e[0] == '0') ? 0 : 1;
        g_fused_df_mode.store(m, std::memory_order_relaxed);
    }
    return m;
}

static std::atomic<int> g_diag_fold_mode{-1};

static std::atomic<int> g_adj_groups_mode{-1};

int adj_phase_groups_enabled() {
    int m = g_adj_groups_mode.load(std::memory_order_relaxed);
    if (m < 0) {
        const char *e = std::getenv("LGPU_ADJ_GROUPS");
        m = (e && e[0] == '0') ? 0 : 1;
        g_adj_groups_mode.store(m, std::memory_order_relaxed);
    }
    return m;
}

int fused_diag_fold_enabled() {
    int m = g_diag_fold_mode.load(std::memory_order_relaxed);
    if (m < 0) {
        const char *e = std::getenv("LGPU_DIAG_FOLD");
        m = (e && (e[0] == '0' || e[0] == '1')) ? e[0] - '0' : 2;
        g_diag_fold_mode.store(m, std::memory_order_relaxed);
    }
    return m;
}

static std::atomic<int> g_tc_mode{-1};

int tc_enabled() {
    int m = g_tc_mode.load(std::memory_order_relaxed);
    if (m < 0) {
        const char *e = std::getenv("LGPU_TC");
        m = (e && e[0] == '0') ? 0 : 1;
        g_tc_mode.store(m, std::memory_order_relaxed);
    }
    return m;
}

int current_device() {
    int d = 0;
    cudaGetDevice(&d);
    return d;
}

int sm_count() {
    static std::mutex mu;
    static std::vector<int> cache;
    const int d = current_device();
    std::lock_guard<std::mutex> lk(mu);
    if (int(cache.size()) <= d) cache.resize(size_t(d) + 1, 0);
    if (cache[size_t(d)] == 0) {
        int v = 0;
        if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, d) != cudaSuccess || v <= 0)
            v = 132;
        cache[size_t(d)] = v;
    }
    return cache[size_t(d)];
}

Holes make_holes(std::vector<int> bits) {
    std::sort(bits.begin(), bits.end());
    Holes h{};
    h.count = int(bits.size());
    for (size_t j = 0; j < bits.size(); j++) h.lo_mask[j] = (uint64_t(1) << bits[j]) - 1;
    return h;
}

lgpu_status_t check_state(const void *sv, uint32_t n, lgpu_dtype_t dt) {
    if (!sv) return fail(LGPU_ERR_INVALID_ARG, "state pointer is null");
    if (n < 1 || n > LGPU_MAX_QUBITS)
        return fail(LGPU_ERR_INVALID_ARG,
                    "number of qubits must be in [1, " + std::to_string(LGPU_MAX_QUBITS) + "], got " +
                        std::to_string(n));
    if (dt != LGPU_C64 && dt != LGPU_C128) return fail(LGPU_ERR_INVALID_ARG, "unknown dtype");
    const uintptr_t align = dt == LGPU_C128 ? 16 : 8;
    if (reinterpret_cast<uintptr_t>(sv) % align)
        return fail(LGPU_ERR_INVALID_ARG, "state pointer is not aligned to one amplitude");
    return LGPU_OK;
}

lgpu_status_t check_bits(uint32_t n, uint32_t count, const int32_t *bits, const char *what,
                         std::vector<int> *out) {
    if (count && !bits) return fail(LGPU_ERR_INVALID_ARG, std::string(what) + " array is null");
    for (uint32_t i = 0; i < count; i++) {
        if (bits[i] < 0 || uint32_t(bits[i]) >= n)
            return fail(LGPU_ERR_INVALID_ARG, std::string(what) + " bit " + std::to_string(bits[i]) +
                                                  " out of range for " + std::to_string(n) +
                                                  " qubits");
        if (out) out->push_back(bits[i]);
    }
    return LGPU_OK;
}

// Scratch of a context.  Bytes 0..127 hold the last-block arrival counter of
// the reductions: zero at allocation, put back to zero by the last block of
// every reduction, and never written by anything else (contexts are reused
// across calls and, through the free list, across states).
lgpu_status_t ctx_scratch(lgpu_context_t ctx, size_t bytes, void **out) {
    if (!ctx) return fail(LGPU_ERR_INVALID_ARG, "context is null");
    if (bytes > ctx->scratch_bytes) {
        // Growth is rare (first use of a larger reduction); finish any work
        // that may still read the old scratch before releasing it.
        if (ctx->scratch) {
            LGPU_CUDA_TRY(cudaDeviceSynchronize());
            LGPU_CUDA_TRY(cudaFree(ctx->scratch));
            ctx->scratch = nullptr;
            ctx->scratch_bytes = 0;
        }
        size_t want = std::max<size_t>(bytes, size_t(1) << 20);
        want = (want + 4095) & ~size_t(4095);
        LGPU_CUDA_TRY(cudaMalloc(&ctx->scratch, want));
        LGPU_CUDA_TRY(cudaMemset(ctx->scratch, 0, want));
        ctx->scratch_bytes = want;
    }
    *out = ctx->scratch;
    return LGPU_OK;
}

lgpu_status_t ctx_pinned(lgpu_context_t ctx, size_t bytes, void **out) {
    if (!ctx) return fail(LGPU_ERR_INVALID_ARG, "context is null");
    if (bytes > ctx->pinned_bytes) {
        if (ctx->pinned) {
            LGPU_CUDA_TRY(cudaDeviceSynchronize());
            LGPU_CUDA_TRY(cudaFreeHost(ctx->pinned));
            ctx->pinned = nullptr;
            ctx->pinned_bytes = 0;
        }
        size_t want = std::max<size_t>(bytes, size_t(1) << 16);
        LGPU_CUDA_TRY(cudaMallocHost(&ctx->pinned, want));
        ctx->pinned_bytes = want;
    }
    *out = ctx->pinned;
    return LGPU_OK;
}

lgpu_status_t reduce_scratch(lgpu_context_t ctx, unsigned grid, unsigned nout, ReduceScratch *rs) {
    void *p = nullptr;
    const size_t bytes = 256 + size_t(grid) * nout * sizeof(double2) + nout * sizeof(double2);
    LGPU_TRY(ctx_scratch(ctx, bytes, &p));
    rs->counter = static_cast<unsigned *>(p);
    rs->partials = reinterpret_cast<double2 *>(static_cast<char *>(p) + 256);
    return LGPU_OK;
}

lgpu_status_t deliver(lgpu_context_t ctx, const double2 *src, size_t count, double *out,
                      int out_on_device, cudaStream_t s) {
    if (!out) return fail(LGPU_ERR_INVALID_ARG, "output pointer is null");
    const size_t bytes = count * sizeof(double2);
    if (out_on_device) {
        LGPU_CUDA_TRY(cudaMemcpyAsync(out, src, bytes, cudaMemcpyDeviceToDevice, s));
        return LGPU_OK;
    }
    void *pin = nullptr;
    LGPU_TRY(ctx_pinned(ctx, bytes, &pin));
    LGPU_CUDA_TRY(cudaMemcpyAsync(pin, src, bytes, cudaMemcpyDeviceToHost, s));
    LGPU_CUDA_TRY(cudaStreamSynchronize(s));
    std::memcpy(out, pin, bytes);
    return LGPU_OK;
}

// ---------------------------------------------------------------------------
// Kernels
// ---------------------------------------------------------------------------
// Fill with zero using 16-byte stores, then place one value.
__global__ void fill_zero_kernel(uint4 *p, uint64_t n16) {
    const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
    const uint4 z = make_uint4(0, 0, 0, 0);
    for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n16; i += stride) p[i] = z;
}

template <class T> __global__ void put_one_kernel(cplx_t<T> *sv, uint64_t index, T re, T im) {
    sv[index] = mk<T>(re, im);
}

template <class T>
__global__ void scatter_kernel(cplx_t<T> *sv, const cplx_t<T> *vals, const int64_t *idx,
                               uint64_t count, uint64_t N) {
    const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
    for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < count; i += stride) {
        const int64_t j = idx[i];
        if (j < 0 || uint64_t(j) >= N) continue;  // callers validate indices on the host
        sv[j] = vals[i];
    }
}

template <class T>
__global__ void axpy_kernel(T ar, T ai, const cplx_t<T> *x, cplx_t<T> *y, uint64_t N) {
    const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
    for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < N; i += stride) {
        const cplx_t<T> a = x[i];
        cplx_t<T> b = y[i];
        b.x = fmaT(ar, a.x, b.x);
        b.x = fmaT(-ai, a.y, b.x);
        b.y = fmaT(ar, a.y, b.y);
        b.y = fmaT(ai, a.x, b.y);
        y[i] = b;
    }
}

template <class T> __global__ void scale_kernel(T ar, T ai, cplx_t<T> *x, uint64_t N) {
    const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
    for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < N; i += stride) {
        const cplx_t<T> a = x[i];
        x[i] = mk<T>(ar * a.x - ai * a.y, ar * a.y + ai * a.x);
    }
}

template <class T> struct DotBody {
    const cplx_t<T> *a;
    const cplx_t<T> *b;
    __device__ __forceinline__ void operator()(uint64_t i, double2 *acc) const {
        const cplx_t<T> u = a[i], v = b[i];
        const double ux = u.x, uy = u.y, vx = v.x, vy = v.y;
        acc[0].x = fma(ux, vx, fma(uy, vy, acc[0].x));
        acc[0].y = fma(ux, vy, fma(-uy, vx, acc[0].y));
    }
};

}  // namespace lgpu

using namespace lgpu;

extern "C" {

int lgpu_abi_version(void) { return 1; }

lgpu_status_t lgpu_set_f64_mode(int mode) {
    if (mode != 0 && mode != 1) return fail(LGPU_ERR_INVALID_ARG, "f64 mode must be 0 (native) or 1 (emulated multiplies)");
    g_f64_mode.store(mode, std::memory_order_relaxed);
    return LGPU_OK;
}

int lgpu_get_f64_mode(void) { return f64_mode(); }

lgpu_status_t lgpu_set_stream_mode(int mode) {
    if (mode != 0 && mode != 1) return fail(LGPU_ERR_INVALID_ARG, "stream mode must be 0 or 1");
    g_bulk_mode.store(mode, std::memory_order_relaxed);
    return LGPU_OK;
}

int lgpu_get_stream_mode(void) { return bulk_enabled(); }

lgpu_status_t lgpu_set_tensor_mode(int mode) {
    if (mode != 0 && mode != 1) return fail(LGPU_ERR_INVALID_ARG, "tensor mode must be 0 or 1");
    g_tc_mode.store(mode, std::memory_order_relaxed);
    return LGPU_OK;
}

int lgpu_get_tensor_mode(void) { return tc_enabled(); }

const char *lgpu_last_error_string(void) { return g_last_error.c_str(); }

lgpu_status_t lgpu_device_count(int *count) {
    if (!count) return fail(LGPU_ERR_INVALID_ARG, "count is null");
    cudaError_t e = cudaGetDeviceCount(count);
    if (e != cudaSuccess) {
        *count = 0;
        cudaGetLastError();
        return fail(LGPU_ERR_NO_DEVICE, std::string("no CUDA device: ") + cudaGetErrorString(e));
    }
    return LGPU_OK;
}

lgpu_status_t lgpu_get_device(int *device) {
    if (!device) return fail(LGPU_ERR_INVALID_ARG, "device is null");
    LGPU_CUDA_TRY(cudaGetDevice(device));
    return LGPU_OK;
}

lgpu_status_t lgpu_set_device(int device) {
    LGPU_CUDA_TRY(cudaSetDevice(device));
    return LGPU_OK;
}

lgpu_status_t lgpu_device_arch(int device, int *major, int *minor) {
    if (!major || !minor) return fail(LGPU_ERR_INVALID_ARG, "null output");
    LGPU_CUDA_TRY(cudaDeviceGetAttribute(major, cudaDevAttrComputeCapabilityMajor, device));
    LGPU_CUDA_TRY(cudaDeviceGetAttribute(minor, cudaDevAttrComputeCapabilityMinor, device));
    return LGPU_OK;
}

lgpu_status_t lgpu_device_sm_count(int device, int *sms) {
    if (!sms) return fail(LGPU_ERR_INVALID_ARG, "null output");
    LGPU_CUDA_TRY(cudaDeviceGetAttribute(sms, cudaDevAttrMultiProcessorCount, device));
    return LGPU_OK;
}

lgpu_status_t lgpu_device_reset(void) {
    int dev = 0;
    LGPU_CUDA_TRY(cudaGetDevice(&dev));
    LGPU_CUDA_TRY(cudaDeviceReset());
    // The reset freed every allocation of the old context and unloaded its
    // module: cached addresses and kernel attributes of this device are stale.
    g_reset_epoch.fetch_add(1, std::memory_order_acq_rel);
    forget_device_state(dev);
    return LGPU_OK;
}

lgpu_status_t lgpu_mem_info(size_t *free_bytes, size_t *total_bytes) {
    if (!free_bytes || !total_bytes) return fail(LGPU_ERR_INVALID_ARG, "null output");
    LGPU_CUDA_TRY(cudaMemGetInfo(free_bytes, total_bytes));
    return LGPU_OK;
}

lgpu_status_t lgpu_malloc(void **ptr, size_t bytes) {
    if (!ptr) return fail(LGPU_ERR_INVALID_ARG, "ptr is null");
    *ptr = nullptr;
    if (bytes == 0) return LGPU_OK;
    cudaError_t e = cudaMalloc(ptr, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        *ptr = nullptr;
        return cuda_fail(e, "cudaMalloc");
    }
    return LGPU_OK;
}

lgpu_status_t lgpu_free(void *ptr) {
    if (ptr) LGPU_CUDA_TRY(cudaFree(ptr));
    return LGPU_OK;
}

lgpu_status_t lgpu_malloc_async(void **ptr, size_t bytes, lgpu_stream_t stream) {
    if (!ptr) return fail(LGPU_ERR_INVALID_ARG, "ptr is null");
    *ptr = nullptr;
    if (bytes == 0) return LGPU_OK;
    int dev = 0;
    LGPU_CUDA_TRY(cudaGetDevice(&dev));
    {
        // the process's default pool keeps freed memory for reuse (set once per device)
        static std::mutex mu;
        static bool done[64] = {};
        std::lock_guard<std::mutex> lock(mu);
        if (dev >= 0 && dev < 64 && !done[dev]) {
            cudaMemPool_t pool;
            LGPU_CUDA_TRY(cudaDeviceGetDefaultMemPool(&pool, dev));
            uint64_t keep = ~uint64_t(0);
            LGPU_CUDA_TRY(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep));
            done[dev] = true;
        }
    }
    cudaError_t e = cudaMallocAsync(ptr, bytes, reinterpret_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) {
        cudaGetLastError();
        *ptr = nullptr;
        return cuda_fail(e, "cudaMallocAsync");
    }
    return LGPU_OK;
}

lgpu_status_t lgpu_free_async(void *ptr, lgpu_stream_t stream) {
    if (ptr) LGPU_CUDA_TRY(cudaFreeAsync(ptr, reinterpret_cast<cudaStream_t>(stream)));
    return LGPU_OK;
}

lgpu_status_t lgpu_host_alloc_pinned(void **ptr, size_t bytes) {
    if (!ptr) return fail(LGPU_ERR_INVALID_ARG, "ptr is null");
    LGPU_CUDA_TRY(cudaMallocHost(ptr, bytes));
    return LGPU_OK;
}

lgpu_status_t lgpu_host_free_pinned(void *ptr) {
    if (ptr) LGPU_CUDA_TRY(cudaFreeHost(ptr));
    return LGPU_OK;
}

lgpu_status_t lgpu_memcpy(void *dst, const void *src, size_t bytes, lgpu_copy_kind_t kind, int async,
                          lgpu_stream_t stream) {
    if (bytes == 0) return LGPU_OK;
    if (!dst || !src) return fail(LGPU_ERR_INVALID_ARG, "null pointer in memcpy");
    cudaMemcpyKind k = kind == LGPU_H2D   ? cudaMemcpyHostToDevice
                       : kind == LGPU_D2H ? cudaMemcpyDeviceToHost
                                          : cudaMemcpyDeviceToDevice;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    LGPU_CUDA_TRY(cudaMemcpyAsync(dst, src, bytes, k, s));
    if (!async) LGPU_CUDA_TRY(cudaStreamSynchronize(s));
    return LGPU_OK;
}

lgpu_status_t lgpu_memset(void *dst, int value, size_t bytes, lgpu_stream_t stream) {
    if (bytes == 0) return LGPU_OK;
    LGPU_CUDA_TRY(cudaMemsetAsync(dst, value, bytes, reinterpret_cast<cudaStream_t>(stream)));
    return LGPU_OK;
}

lgpu_status_t lgpu_stream_create(lgpu_stream_t *stream) {
    if (!stream) return fail(LGPU_ERR_INVALID_ARG, "stream is null");
    cudaStream_t s;
    LGPU_CUDA_TRY(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    *stream = reinterpret_cast<lgpu_stream_t>(s);
    return LGPU_OK;
}

lgpu_status_t lgpu_stream_destroy(lgpu_stream_t stream) {
    if (stream) LGPU_CUDA_TRY(cudaStreamDestroy(reinterpret_cast<cudaStream_t>(stream)));
    return LGPU_OK;
}

lgpu_status_t lgpu_stream_sync(lgpu_stream_t stream) {
    LGPU_CUDA_TRY(cudaStreamSynchronize(reinterpret_cast<cudaStream_t>(stream)));
    return LGPU_OK;
}

lgpu_status_t lgpu_peer_access_all(void) {
    int n = 0;
    LGPU_CUDA_TRY(cudaGetDeviceCount(&n));
    for (int i = 0; i < n; i++) {
        cudaError_t e = cudaDeviceEnablePeerAccess(i, 0);
        if (e != cudaSuccess) cudaGetLastError();  // self or unsupported pair: ignore
    }
    return LGPU_OK;
}

struct lgpu_graph_s {
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
};

lgpu_status_t lgpu_graph_begin(lgpu_stream_t stream) {
    LGPU_CUDA_TRY(cudaStreamBeginCapture(reinterpret_cast<cudaStream_t>(stream), cudaStreamCaptureModeThreadLocal));
    return LGPU_OK;
}

lgpu_status_t lgpu_graph_end(lgpu_stream_t stream, lgpu_graph_t *graph) {
    if (!graph) return fail(LGPU_ERR_INVALID_ARG, "graph is null");
    auto *g = new (std::nothrow) lgpu_graph_s();
    if (!g) return fail(LGPU_ERR_OOM, "host allocation of graph failed");
    cudaError_t e = cudaStreamEndCapture(reinterpret_cast<cudaStream_t>(stream), &g->graph);
    if (e != cudaSuccess) {
        delete g;
        return cuda_fail(e, "cudaStreamEndCapture");
    }
    e = cudaGraphInstantiate(&g->exec, g->graph, 0);
    if (e != cudaSuccess) {
        cudaGraphDestroy(g->graph);
        delete g;
        return cuda_fail(e, "cudaGraphInstantiate");
    }
    *graph = g;
    return LGPU_OK;
}

lgpu_status_t lgpu_graph_launch(lgpu_graph_t graph, lgpu_stream_t stream) {
    if (!graph) return fail(LGPU_ERR_INVALID_ARG, "graph is null");
    LGPU_CUDA_TRY(cudaGraphLaunch(graph->exec, reinterpret_cast<cudaStream_t>(stream)));
    return LGPU_OK;
}

lgpu_status_t lgpu_graph_destroy(lgpu_graph_t graph) {
    if (!graph) return LGPU_OK;
    if (graph->exec) cudaGraphExecDestroy(graph->exec);
    if (graph->graph) cudaGraphDestroy(graph->graph);
    delete graph;
    return LGPU_OK;
}

lgpu_status_t lgpu_context_create(int device, lgpu_context_t *ctx) {
    if (!ctx) return fail(LGPU_ERR_INVALID_ARG, "ctx is null");
    auto *c = new (std::nothrow) lgpu_context_s();
    if (!c) return fail(LGPU_ERR_OOM, "host allocation of context failed");
    c->device = device;
    *ctx = c;
    return LGPU_OK;
}

lgpu_status_t lgpu_context_destroy(lgpu_context_t ctx) {
    if (!ctx) return LGPU_OK;
    if (ctx->scratch || ctx->pinned) cudaDeviceSynchronize();
    if (ctx->scratch) cudaFree(ctx->scratch);
    if (ctx->pinned) cudaFreeHost(ctx->pinned);
    delete ctx;
    return LGPU_OK;
}

static std::mutex g_ctx_pool_mu;
static std::vector<lgpu_context_t> g_ctx_pool[64];

lgpu_status_t lgpu_context_acquire(int device, lgpu_context_t *ctx) {
    if (!ctx) return fail(LGPU_ERR_INVALID_ARG, "ctx is null");
    if (device >= 0 && device < 64) {
        std::lock_guard<std::mutex> lock(g_ctx_pool_mu);
        auto &free_list = g_ctx_pool[device];
        if (!free_list.empty()) {
            *ctx = free_list.back();
            free_list.pop_back();
            return LGPU_OK;
        }
    }
    return lgpu_context_create(device, ctx);
}

lgpu_status_t lgpu_context_release(lgpu_context_t ctx) {
    if (!ctx) return LGPU_OK;
    if (ctx->device >= 0 && ctx->device < 64) {
        std::lock_guard<std::mutex> lock(g_ctx_pool_mu);
        auto &free_list = g_ctx_pool[ctx->device];
        if (free_list.size() < 256) {
            free_list.push_back(ctx);
            return LGPU_OK;
        }
    }
    return lgpu_context_destroy(ctx);
}

lgpu_status_t lgpu_context_reserve(lgpu_context_t ctx, size_t bytes) {
    void *p = nullptr;
    return ctx_scratch(ctx, bytes, &p);
}

lgpu_status_t lgpu_set_basis(void *sv, uint32_t n, lgpu_dtype_t dt, uint64_t index, double re,
                             double im, lgpu_stream_t stream) {
    LGPU_TRY(check_state(sv, n, dt));
    const uint64_t N = uint64_t(1) << n;
    if (index >= N) return fail(LGPU_ERR_INVALID_ARG, "basis index out of range");
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const uint64_t bytes = N * amp_bytes(dt);
    if (bytes % 16 == 0) {
        const uint64_t n16 = bytes / 16;
        fill_zero_kernel<<<grid_for(n16, 256, 4), 256, 0, s>>>(static_cast<uint4 *>(sv), n16);
        LGPU_CHECK_LAUNCH();
    } else {
        LGPU_CUDA_TRY(cudaMemsetAsync(sv, 0, bytes, s));
    }
    if (dt == LGPU_C128)
        put_one_kernel<double><<<1, 1, 0, s>>>(static_cast<double2 *>(sv), index, re, im);
    else
        put_one_kernel<float><<<1, 1, 0, s>>>(static_cast<float2 *>(sv), index, float(re), float(im));
    LGPU_CHECK_LAUNCH();
    return LGPU_OK;
}

lgpu_status_t lgpu_scatter(void *sv, uint32_t n, lgpu_dtype_t dt, const void *values,
                           const int64_t *indices, uint64_t count, int zero_first,
                           lgpu_stream_t stream) {
    LGPU_TRY(check_state(sv, n, dt));
    if (count && (!values || !indices)) return fail(LGPU_ERR_INVALID_ARG, "null values/indices");
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const uint64_t N = uint64_t(1) << n;
    if (zero_first) {
        const uint64_t bytes = N * amp_bytes(dt);
        if (bytes % 16 == 0) {
            fill_zero_kernel<<<grid_for(bytes / 16, 256, 4), 256, 0, s>>>(static_cast<uint4 *>(sv),
                                                                           bytes / 16);
            LGPU_CHECK_LAUNCH();
        } else {
            LGPU_CUDA_TRY(cudaMemsetAsync(sv, 0, bytes, s));
        }
    }
    if (count == 0) return LGPU_OK;
    const unsigned g = grid_for(count, 256, 1);
    if (dt == LGPU_C128)
        scatter_kernel<double><<<g, 256, 0, s>>>(static_cast<double2 *>(sv),
                                                 static_cast<const double2 *>(values), indices, count,
                                                 N);
    else
        scatter_kernel<float><<<g, 256, 0, s>>>(static_cast<float2 *>(sv),
                                                static_cast<const float2 *>(values), indices, count, N);
    LGPU_CHECK_LAUNCH();
    return LGPU_OK;
}

lgpu_status_t lgpu_copy(void *dst, const void *src, uint32_t n, lgpu_dtype_t dt, lgpu_stream_t stream) {
    LGPU_TRY(check_state(dst, n, dt));
    LGPU_TRY(check_state(src, n, dt));
    if (dst == src) return LGPU_OK;
    LGPU_CUDA_TRY(cudaMemcpyAsync(dst, src, (uint64_t(1) << n) * amp_bytes(dt),
                                  cudaMemcpyDeviceToDevice, reinterpret_cast<cudaStream_t>(stream)));
    return LGPU_OK;
}

lgpu_status_t lgpu_axpy(double alpha_re, double alpha_im, const void *x, void *y, uint32_t n,
                        lgpu_dtype_t dt, lgpu_stream_t stream) {
    LGPU_TRY(check_state(x, n, dt));
    LGPU_TRY(check_state(y, n, dt));
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const uint64_t N = uint64_t(1) << n;
    const unsigned g = grid_for(N, 256, 4);
    if (dt == LGPU_C128)
        axpy_kernel<double><<<g, 256, 0, s>>>(alpha_re, alpha_im, static_cast<const double2 *>(x),
                                              static_cast<double2 *>(y), N);
    else
        axpy_kernel<float><<<g, 256, 0, s>>>(float(alpha_re), float(alpha_im),
                                             static_cast<const float2 *>(x), static_cast<float2 *>(y),
                                             N);
    LGPU_CHECK_LAUNCH();
    return LGPU_OK;
}

lgpu_status_t lgpu_scale(double alpha_re, double alpha_im, void *x, uint32_t n, lgpu_dtype_t dt,
                         lgpu_stream_t stream) {
    LGPU_TRY(check_state(x, n, dt));
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const uint64_t N = uint64_t(1) << n;
    const unsigned g = grid_for(N, 256, 4);
    if (dt == LGPU_C128)
        scale_kernel<double><<<g, 256, 0, s>>>(alpha_re, alpha_im, static_cast<double2 *>(x), N);
    else
        scale_kernel<float><<<g, 256, 0, s>>>(float(alpha_re), float(alpha_im),
                                              static_cast<float2 *>(x), N);
    LGPU_CHECK_LAUNCH();
    return LGPU_OK;
}

lgpu_status_t lgpu_dot(lgpu_context_t ctx, const void *a, const void *b, uint32_t n,
                       lgpu_dtype_t dt, double *out, int out_on_device, lgpu_stream_t stream) {
    LGPU_TRY(check_state(a, n, dt));
    LGPU_TRY(check_state(b, n, dt));
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const uint64_t N = uint64_t(1) << n;
    const unsigned g = reduce_grid(N);
    ReduceScratch rs;
    LGPU_TRY(reduce_scratch(ctx, g, 1, &rs));
    double2 *res = rs.partials + size_t(g);
    if (dt == LGPU_C128) {
        DotBody<double> body{static_cast<const double2 *>(a), static_cast<const double2 *>(b)};
        reduce_kernel<1, uint64_t><<<g, kReduceBlock, 0, s>>>(body, N, rs.partials, rs.counter, res);
    } else {
        DotBody<float> body{static_cast<const float2 *>(a), static_cast<const float2 *>(b)};
        reduce_kernel<1, uint64_t><<<g, kReduceBlock, 0, s>>>(body, N, rs.partials, rs.counter, res);
    }
    LGPU_CHECK_LAUNCH();
    return deliver(ctx, res, 1, out, out_on_device, s);
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Allocation-free inner product
// ---------------------------------------------------------------------------
// lgpu_dot_static runs the same reduction as lgpu_dot (same grid, same fixed
// summation order, hence the same bits) but takes its scratch from the
// file-scope device array below instead of a context, and copies a host
// result straight into the caller's buffer.  It calls no cudaMalloc,
// cudaMallocHost, cudaFree or other allocating routine.
//
// Scratch layout: [arrival counter, 256 B][partials: grid x double2]
// [result: double2].  Only the counter must start at zero: static device
// memory is zero when the module loads, and the reduction's last block writes
// the counter back to zero.  The partials and the result are written before
// they are read.
//
// Set-up: the device address of the array is looked up once per device
// (cudaGetSymbolAddress with that device current) on the first call made
// with that device current, and cached.  That lookup may load the module on
// the device, so the first call on each device belongs before any stream
// capture.
//
// One array per device serves every call: two calls that can run at the same
// time on one device (different streams, or host threads without ordering)
// race on it and may return garbage.  Callers order them (one stream, or a
// synchronisation between calls).
namespace lgpu {

constexpr size_t kStaticScratchBytes = size_t(32) << 10;  // 32 KiB per device
__device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

constexpr int kStaticMaxDevices = 64;
static std::atomic<void *> g_static_ptr[kStaticMaxDevices];
static std::mutex g_static_mu;

lgpu_status_t static_scratch(cudaStream_t stream, void **out) {
    int dev = 0;
    LGPU_CUDA_TRY(cudaGetDevice(&dev));
    int stream_dev = dev;
    // The legacy and per-thread default streams (handles 0, 1, 2) follow the
    // current device.
    if (reinterpret_cast<uintptr_t>(stream) > 2) LGPU_CUDA_TRY(cudaStreamGetDevice(stream, &stream_dev));
    if (stream_dev != dev)
        return fail(LGPU_ERR_INVALID_ARG, "lgpu_dot_static: the stream belongs to device " +
                                              std::to_string(stream_dev) + " but device " + std::to_string(dev) +
                                              " is current; make the stream's device current");
    if (dev < 0 || dev >= kStaticMaxDevices)
        return fail(LGPU_ERR_UNSUPPORTED, "lgpu_dot_static: device ordinal " + std::to_string(dev) +
                                              " is beyond the " + std::to_string(kStaticMaxDevices) +
                                              " devices it keeps scratch addresses for");
    void *p = g_static_ptr[dev].load(std::memory_order_acquire);
    if (!p) {
        std::lock_guard<std::mutex> lock(g_static_mu);
        p = g_static_ptr[dev].load(std::memory_order_relaxed);
        if (!p) {
            LGPU_CUDA_TRY(cudaGetSymbolAddress(&p, g_static_scratch));
            g_static_ptr[dev].store(p, std::memory_order_release);
        }
    }
    *out = p;
    return LGPU_OK;
}

void forget_device_state(int dev) {
    if (dev < 0 || dev >= kStaticMaxDevices) return;
    {
        std::lock_guard<std::mutex> lock(g_static_mu);
        g_static_ptr[dev].store(nullptr, std::memory_order_release);
    }
    std::lock_guard<std::mutex> lock(g_ctx_pool_mu);
    // The pooled contexts' scratch and pinned buffers died with the reset:
    // drop the host records without freeing through the new context.
    for (lgpu_context_t c : g_ctx_pool[dev]) delete c;
    g_ctx_pool[dev].clear();
}

}  // namespace lgpu

extern "C" {

size_t lgpu_dot_static_scratch_bytes(void) { return kStaticScratchBytes; }

lgpu_status_t lgpu_dot_static(const void *a, const void *b, uint32_t n, lgpu_dtype_t dt, double *out,
                              int out_on_device, lgpu_stream_t stream) {
    LGPU_TRY(check_state(a, n, dt));
    LGPU_TRY(check_state(b, n, dt));
    if (!out) return fail(LGPU_ERR_INVALID_ARG, "output pointer is null");
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const uint64_t N = uint64_t(1) << n;
    const unsigned g = reduce_grid(N);
    const size_t need = 256 + (size_t(g) + 1) * sizeof(double2);
    if (need > kStaticScratchBytes)
        return fail(LGPU_ERR_INVALID_ARG, "lgpu_dot_static: the reduction over 2^" + std::to_string(n) +
                                              " amplitudes uses " + std::to_string(g) + " blocks and needs " +
                                              std::to_string(need) + " bytes of scratch; the static scratch holds " +
                                              std::to_string(kStaticScratchBytes) + " bytes");
    void *base = nullptr;
    LGPU_TRY(static_scratch(s, &base));
    unsigned *counter = static_cast<unsigned *>(base);
    double2 *partials = reinterpret_cast<double2 *>(static_cast<char *>(base) + 256);
    double2 *res = partials + size_t(g);
    if (dt == LGPU_C128) {
        DotBody<double> body{static_cast<const double2 *>(a), static_cast<const double2 *>(b)};
        reduce_kernel<1, uint64_t><<<g, kReduceBlock, 0, s>>>(body, N, partials, counter, res);
    } else {
        DotBody<float> body{static_cast<const float2 *>(a), static_cast<const float2 *>(b)};
        reduce_kernel<1, uint64_t><<<g, kReduceBlock, 0, s>>>(body, N, partials, counter, res);
    }
    LGPU_CHECK_LAUNCH();
    if (out_on_device) {
        LGPU_CUDA_TRY(cudaMemcpyAsync(out, res, sizeof(double2), cudaMemcpyDeviceToDevice, s));
        return LGPU_OK;
    }
    LGPU_CUDA_TRY(cudaMemcpyAsync(out, res, sizeof(double2), cudaMemcpyDeviceToHost, s));
    LGPU_CUDA_TRY(cudaStreamSynchronize(s));
    return LGPU_OK;
}

}  // extern "C"
