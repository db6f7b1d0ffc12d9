// Internal helpers shared by the liblgpu_gb300 translation units.
#pragma once

#include <atomic>

#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "lgpu.h"

namespace lgpu {

// ---------------------------------------------------------------------------
// Error plumbing (thread-local last error, status codes)
// ---------------------------------------------------------------------------
void set_error(const std::string &msg);
lgpu_status_t fail(lgpu_status_t st, const std::string &msg);
lgpu_status_t cuda_fail(cudaError_t e, const char *what);

#define LGPU_CUDA_TRY(expr)                                                                   \
    do {                                                                                       \
        cudaError_t _e = (expr);                                                               \
        if (_e != cudaSuccess) return ::lgpu::cuda_fail(_e, #expr);                             \
    } while (0)

#define LGPU_CHECK_LAUNCH()                                                                    \
    do {                                                                                       \
        cudaError_t _e = cudaGetLastError();                                                   \
        if (_e != cudaSuccess) return ::lgpu::cuda_fail(_e, "kernel launch");                   \
    } while (0)

#define LGPU_TRY(expr)                                                                         \
    do {                                                                                       \
        lgpu_status_t _s = (expr);                                                             \
        if (_s != LGPU_OK) return _s;                                                          \
    } while (0)

// ---------------------------------------------------------------------------
// Device properties (cached per device)
// ---------------------------------------------------------------------------
int sm_count();          // SMs of the current device
int current_device();
// complex128 arithmetic mode: 0 = native FP64, 1 = FP64 FMA + integer-pipe
// multiplies (lgpu_f64emu.cuh).  Process-wide; see lgpu_set_f64_mode().
int f64_mode();
// complex128 fused blocks run 1-target bodies in float-float arithmetic when 1
// (default, with f64_mode() == 1); the integer-pipe bodies when 0
// (environment LGPU_FUSED_DF=0).
int fused_df_enabled();
// Folding of diagonal gates into phase tables in float-float fused blocks:
// 2 (default) = fold, with dense 1-target gates split into diagonals and a
// real rotation where that pays; 1 = fold without splits; 0 = off
// (environment LGPU_DIAG_FOLD).
int fused_diag_fold_enabled();
// Phase groups in the adjoint blocks (uncontrolled diagonal steps share one
// overlap product and one phase table): 1 (default) = on, 0 = off
// (environment LGPU_ADJ_GROUPS).
int adj_phase_groups_enabled();
// Uncontrolled 1-target gates use the bulk-copy pipelined kernel when 1
// (default); the grid-stride kernel when 0.  See lgpu_set_stream_mode().
int bulk_enabled();
// Dense 6-target complex64 gates on the six lowest state bits run on the
// tensor cores (tcgen05) when 1 (default); the shared-memory FP32 kernel when
// 0 (environment LGPU_TC=0).  See lgpu_set_tensor_mode().
int tc_enabled();
// device error flag of the batched kernel's bounded waits (lgpu_batch.cu)
lgpu_status_t batch_error_fetch(unsigned *v, bool reset);
// Per-stream error words of the bounded waits: kernels launched on stream s
// receive *out (a device address on the current device) and set it on a
// time-out; lgpu_stream_error reads it.
constexpr int kErrSlots = 256;
lgpu_status_t stream_error_ptr(cudaStream_t s, unsigned **out);

// ---------------------------------------------------------------------------
// Scratch context
// ---------------------------------------------------------------------------
}  // namespace lgpu

struct lgpu_context_s {
    int device = 0;
    void *scratch = nullptr;
    size_t scratch_bytes = 0;
    // host-pinned staging for small results
    void *pinned = nullptr;
    size_t pinned_bytes = 0;
};

namespace lgpu {

lgpu_status_t ctx_scratch(lgpu_context_t ctx, size_t bytes, void **out);
lgpu_status_t ctx_pinned(lgpu_context_t ctx, size_t bytes, void **out);

// ---------------------------------------------------------------------------
// Complex amplitude types
// ---------------------------------------------------------------------------
template <class T> struct vec2;
template <> struct vec2<double> { using type = double2; };
template <> struct vec2<float> { using type = float2; };
template <class T> using cplx_t = typename vec2<T>::type;

template <class T> __host__ __device__ __forceinline__ cplx_t<T> mk(T re, T im) {
    cplx_t<T> r;
    r.x = re;
    r.y = im;
    return r;
}
template <class T>
__host__ __device__ __forceinline__ cplx_t<T> cmul(cplx_t<T> a, cplx_t<T> b) {
    return mk<T>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double fmaT(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ float fmaT(float a, float b, float c) { return __fmaf_rn(a, b, c); }

// acc + a*b
template <class T>
__device__ __forceinline__ cplx_t<T> cfma(cplx_t<T> a, cplx_t<T> b, cplx_t<T> acc) {
    acc.x = fmaT(a.x, b.x, acc.x);
    acc.x = fmaT(-a.y, b.y, acc.x);
    acc.y = fmaT(a.x, b.y, acc.y);
    acc.y = fmaT(a.y, b.x, acc.y);
    return acc;
}

// Unaligned-safe vector loads/stores of one amplitude.
template <class T> __device__ __forceinline__ cplx_t<T> ld(const cplx_t<T> *p) { return *p; }
template <class T> __device__ __forceinline__ void st(cplx_t<T> *p, cplx_t<T> v) { *p = v; }

// ---------------------------------------------------------------------------
// Index insertion: spread the bits of a group index g around a sorted list of
// "hole" bit positions (each hole receives a 0).
// ---------------------------------------------------------------------------
constexpr int kMaxHoles = LGPU_MAX_DENSE_TARGETS + LGPU_MAX_CONTROLS + 2;

struct Holes {
    int count;
    uint64_t lo_mask[kMaxHoles];  // (1 << pos) - 1 for each hole, ascending positions
};

template <class I> __device__ __forceinline__ I insert_holes(I g, const Holes &h) {
#pragma unroll 4
    for (int j = 0; j < h.count; j++) {
        const I lo = I(h.lo_mask[j]);
        g = ((g & ~lo) << 1) | (g & lo);
    }
    return g;
}

// Host: build the hole list from bit positions (must be distinct).
Holes make_holes(std::vector<int> bits);

// ---------------------------------------------------------------------------
// Launch geometry: persistent-style grids sized as a multiple of the SM count.
// ---------------------------------------------------------------------------
inline unsigned grid_for(uint64_t work_items, unsigned block, unsigned items_per_thread,
                         unsigned max_blocks_per_sm = 8) {
    const uint64_t per_block = uint64_t(block) * items_per_thread;
    uint64_t blocks = (work_items + per_block - 1) / per_block;
    const uint64_t cap = uint64_t(sm_count()) * max_blocks_per_sm;
    if (blocks > cap) blocks = cap;
    if (blocks < 1) blocks = 1;
    return unsigned(blocks);
}

// ---------------------------------------------------------------------------
// Argument validation helpers
// ---------------------------------------------------------------------------
lgpu_status_t check_state(const void *sv, uint32_t n, lgpu_dtype_t dt);
lgpu_status_t check_bits(uint32_t n, uint32_t count, const int32_t *bits, const char *what,
                         std::vector<int> *out);
inline size_t amp_bytes(lgpu_dtype_t dt) { return dt == LGPU_C128 ? 16 : 8; }

// ---------------------------------------------------------------------------
// Deterministic block reduction of a double2 (FP64) into per-block partials
// followed by a last-block-done final sum in fixed order.
// ---------------------------------------------------------------------------
template <int BLOCK>
__device__ __forceinline__ double2 block_reduce_d2(double2 v, double2 *smem /* BLOCK/32 */) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
        v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) smem[warp] = v;
    __syncthreads();
    if (warp == 0) {
        v = (lane < BLOCK / 32) ? smem[lane] : make_double2(0.0, 0.0);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
            v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
        }
    }
    return v;  // valid in thread 0
}

// Finish: write partial of this block; the last block sums all partials in
// index order into *out and re-arms the counter.  `nout` interleaved outputs
// per block (partials laid out [block][nout]).
__device__ __forceinline__ bool last_block_arrive(unsigned *counter) {
    __shared__ bool is_last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned prev = atomicAdd(counter, 1u);
        is_last = (prev == gridDim.x - 1);
    }
    __syncthreads();
    return is_last;
}

// Number of lgpu_device_reset calls so far.  A reset destroys the device's
// context: kernel attributes set with cudaFuncSetAttribute, module addresses
// and allocations are gone, so every per-device cache of them is tagged with
// the count at which it was filled and refilled when the count has moved.
unsigned reset_epoch();

// Opt `kernel` in to `smem` bytes of dynamic shared memory on the current
// device, once per (kernel, device, size, reset epoch).  cudaFuncSetAttribute
// is not a stream operation: the first launch of each size runs outside any
// stream capture.  `cache` is the kernel's own array (a static of the caller)
// holding (epoch << 40) | bytes; concurrent host threads may race to set the
// same value, which is harmless.
inline lgpu_status_t ensure_smem(const void *kernel, size_t smem, std::atomic<size_t> (&cache)[64]) {
    if (smem <= 48 * 1024) return LGPU_OK;
    int dev = 0;
    LGPU_CUDA_TRY(cudaGetDevice(&dev));
    const bool cached = dev >= 0 && dev < 64;
    const size_t epoch = size_t(reset_epoch()) << 40, bytes_mask = (size_t(1) << 40) - 1;
    if (cached) {
        const size_t v = cache[dev].load(std::memory_order_acquire);
        if ((v & ~bytes_mask) == epoch && smem <= (v & bytes_mask)) return LGPU_OK;
    }
    const cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute");
    if (cached) {
        size_t cur = cache[dev].load(std::memory_order_relaxed);
        while (((cur & ~bytes_mask) != epoch || (cur & bytes_mask) < smem) &&
               !cache[dev].compare_exchange_weak(cur, epoch | smem, std::memory_order_release)) {
        }
    }
    return LGPU_OK;
}

// 8-point Walsh-Hadamard transform W[h] = sum_j (-1)^popc(j & h) x_j (in
// place, Sylvester order) and a branch-free pick of W[h] for a runtime h.
template <class A> __device__ __forceinline__ void wht8(A (&x)[8]) {
#pragma unroll
    for (int len = 1; len < 8; len <<= 1)
#pragma unroll
        for (int i = 0; i < 8; i++)
            if (!(i & len)) {
                const A u = x[i], v = x[i | len];
                x[i] = u + v;
                x[i | len] = u - v;
            }
}

template <class A> __device__ __forceinline__ A sel8(const A (&x)[8], uint32_t h) {
    const A s0 = (h & 1u) ? x[1] : x[0], s1 = (h & 1u) ? x[3] : x[2];
    const A s2 = (h & 1u) ? x[5] : x[4], s3 = (h & 1u) ? x[7] : x[6];
    const A u0 = (h & 2u) ? s1 : s0, u1 = (h & 2u) ? s3 : s2;
    return (h & 4u) ? u1 : u0;
}

}  // namespace lgpu
