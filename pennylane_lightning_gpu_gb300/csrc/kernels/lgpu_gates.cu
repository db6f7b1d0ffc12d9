// liblgpu_gb300: gate application.
//
//  * gate1_kernel     one target bit, streaming pairs (i, i | 1<<t) with
//                     128-bit loads per amplitude (c128) and several pairs in
//                     flight per thread; the body is chosen on the host from
//                     the matrix structure so that FP64 work is minimal.
//  * phase_kernel     multiply the amplitudes whose bits match a mask by one
//                     phase (PhaseShift, S, T, Z, CZ, controlled phases):
//                     only the touched half/quarter of the state is streamed.
//  * gatek_kernel     dense 2^t x 2^t (t = 2..5) with the matrix in the
//                     kernel-parameter bank (uniform broadcast reads).
//  * gatebig_kernel   dense t = 6..12, matrix in global memory, groups staged
//                     in shared memory.
//  * pauli_rot_kernel exp(i angle P) for Pauli words, pairwise (i, i^flip).
//  * fused_kernel     a block of 1/2-target gates applied to shared-memory
//                     tiles of 2^k amplitudes: one HBM pass for many gates.
#include <algorithm>
#include <complex>
#include <cstring>
#include <memory>
#include <mutex>
#include <unordered_map>

#include "lgpu_bodies.cuh"
#include "lgpu_df2.cuh"
#include "lgpu_df64.cuh"
#include "lgpu_f64emu.cuh"
#include "lgpu_fused_plan.h"
#include "lgpu_internal.cuh"

namespace lgpu {

constexpr int kGateBlock = 256;

// ITEMS pairs per thread in flight: all loads are issued before any math.
template <class T, class I, int BODY, int ITEMS, bool EMU>
__global__ void __launch_bounds__(kGateBlock)
    gate1_kernel(cplx_t<T> *__restrict__ sv, const G1Params<T, I> p, const unsigned nstates,
                 cplx_t<T> *const *__restrict__ svs) {
    using C = cplx_t<T>;
    C *s = nstates ? svs[blockIdx.y] : sv;
    T m[8];
#pragma unroll
    for (int k = 0; k < 8; k++) m[k] = p.m[k];
    KConst kc[4];
#pragma unroll
    for (int k = 0; k < 4; k++) kc[k] = p.k[k];
    const I stride = I(gridDim.x) * kGateBlock;
    for (I g = I(blockIdx.x) * kGateBlock + threadIdx.x; g < p.ngroups; g += stride * ITEMS) {
        C a0[ITEMS], a1[ITEMS];
        I i0[ITEMS];
#pragma unroll
        for (int k = 0; k < ITEMS; k++) {
            const I gk = g + I(k) * stride;
            i0[k] = (gk < p.ngroups) ? (insert_holes<I>(gk, p.holes) | p.cset) : I(0);
        }
#pragma unroll
        for (int k = 0; k < ITEMS; k++) {
            if (g + I(k) * stride < p.ngroups) {
                a0[k] = __ldcs(&s[i0[k]]);
                a1[k] = __ldcs(&s[i0[k] | p.tbit]);
            }
        }
#pragma unroll
        for (int k = 0; k < ITEMS; k++) body1_sel<T, BODY, EMU>(m, kc, a0[k], a1[k]);
#pragma unroll
        for (int k = 0; k < ITEMS; k++) {
            if (g + I(k) * stride < p.ngroups) {
                __stcs(&s[i0[k]], a0[k]);
                __stcs(&s[i0[k] | p.tbit], a1[k]);
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Bulk-copy pipelined variant for uncontrolled 1-target gates.
//
// Persistent CTAs (one per SM) stream tiles of 2*CH amplitudes through a ring
// of STAGES shared-memory buffers.  Loads are 1-D cp.async.bulk copies (TMA
// engine) that complete on an mbarrier with a transaction count; stores are
// bulk copies back to global memory.  For a target bit t >= log2(CH) a tile
// is two runs of CH amplitudes 2^t apart (bit t = 0 and 1); otherwise a tile
// is one contiguous run of 2*CH amplitudes with the pairs interleaved.  Every
// wait is bounded: on time-out the CTA records an error in
// g_lgpu_device_error and leaves.
// ---------------------------------------------------------------------------
__device__ unsigned int g_lgpu_device_error = 0;
// One error word per stream (slot); kernels with bounded waits receive the
// address of their launch stream's word and set it besides the device-wide flag.
__device__ unsigned int g_lgpu_stream_error[kErrSlots];

// Mark a timed-out wait: the launch stream's word and the device-wide flag.
__device__ __forceinline__ void report_timeout(unsigned *err) {
    if (err) atomicOr(err, 1u);
    atomicOr(&g_lgpu_device_error, 1u);
}

constexpr int kBulkThreads = 512;
constexpr int kBulkStages = 3;
constexpr uint32_t kWaitLimit = 1u << 24;  // try_wait polls before giving up

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Self-test of the bounded waits: one CTA arms an mbarrier with a transaction
// count that no copy will deliver (a flag nothing sets) and waits with the
// streaming kernels' bounded spin; it gives up after `spin_limit` polls and
// records the time-out in g_lgpu_device_error, as they do.
__global__ void wait_selftest_kernel(uint32_t spin_limit, unsigned *err) {
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (threadIdx.x == 0) mbar_expect_tx(&bar, 16);  // 16 bytes that never arrive
    __syncthreads();
    uint32_t spins = 0;
    bool timed_out = false;
    while (!mbar_try_wait(&bar, 0)) {
        if (++spins > spin_limit) {
            timed_out = true;
            break;
        }
    }
    if (__syncthreads_or(timed_out) && threadIdx.x == 0) report_timeout(err);
}

__device__ __forceinline__ void bulk_load(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}
__device__ __forceinline__ void bulk_store(void *dst, const void *src, uint32_t bytes) {
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst), "r"(smem_u32(src)),
                 "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_read1() { asm volatile("cp.async.bulk.wait_group.read 1;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }
__device__ __forceinline__ void fence_async_shared() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

template <class T> struct BulkParams {
    unsigned *err;   // the launch stream's error word
    uint64_t ntiles;
    int t;           // target bit
    int ch_log2;     // log2(CH)
    T m[8];
    KConst k[4];
};

template <class T, int BODY, bool EMU>
__global__ void __launch_bounds__(kBulkThreads, 1)
    gate1_bulk_kernel(cplx_t<T> *__restrict__ sv, const BulkParams<T> p) {
    using C = cplx_t<T>;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t full_bar[kBulkStages];
    C *ring = reinterpret_cast<C *>(smem_raw);
    const uint32_t CH = 1u << p.ch_log2;
    const uint32_t half_bytes = CH * uint32_t(sizeof(C));
    const bool split = p.t >= p.ch_log2;
    const uint64_t G = gridDim.x;
    T m[8];
#pragma unroll
    for (int q = 0; q < 8; q++) m[q] = p.m[q];
    KConst kc[4];
#pragma unroll
    for (int q = 0; q < 4; q++) kc[q] = p.k[q];

    // global amplitude index of the start of each half of tile `tile`
    auto tile_base = [&](uint64_t tile) -> uint64_t {
        if (!split) return tile << (p.ch_log2 + 1);
        const int hb = p.t - p.ch_log2;  // bit of the block index that is the target bit
        const uint64_t lo = tile & ((uint64_t(1) << hb) - 1);
        return (((tile >> hb) << (hb + 1)) | lo) << p.ch_log2;
    };
    auto issue_load = [&](uint64_t tile, int s) {
        C *buf = ring + size_t(s) * 2 * CH;
        const uint64_t b0 = tile_base(tile);
        mbar_expect_tx(&full_bar[s], 2 * half_bytes);
        if (split) {
            bulk_load(buf, sv + b0, half_bytes, &full_bar[s]);
            bulk_load(buf + CH, sv + b0 + (uint64_t(1) << p.t), half_bytes, &full_bar[s]);
        } else {
            bulk_load(buf, sv + b0, 2 * half_bytes, &full_bar[s]);
        }
    };
    auto issue_store = [&](uint64_t tile, int s) {
        C *buf = ring + size_t(s) * 2 * CH;
        const uint64_t b0 = tile_base(tile);
        if (split) {
            bulk_store(sv + b0, buf, half_bytes);
            bulk_store(sv + b0 + (uint64_t(1) << p.t), buf + CH, half_bytes);
        } else {
            bulk_store(sv + b0, buf, 2 * half_bytes);
        }
        bulk_commit();
    };

    if (threadIdx.x == 0) {
#pragma unroll
        for (int s = 0; s < kBulkStages; s++) mbar_init(&full_bar[s], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int s = 0; s < kBulkStages; s++) {
            const uint64_t tile = blockIdx.x + uint64_t(s) * G;
            if (tile < p.ntiles) issue_load(tile, s);
        }
    }
    bool failed = false;
    uint64_t j = 0;
    for (;; j++) {
        const uint64_t tile = blockIdx.x + j * G;
        if (tile >= p.ntiles) break;
        const int s = int(j % kBulkStages);
        const uint32_t parity = uint32_t((j / kBulkStages) & 1);
        uint32_t spins = 0;
        bool timed_out = false;
        while (!mbar_try_wait(&full_bar[s], parity)) {
            if (++spins > kWaitLimit) {
                timed_out = true;
                break;
            }
        }
        // Every thread leaves its bounded wait; the CTA then decides together.
        failed = __syncthreads_or(timed_out) != 0;
        if (failed) {
            if (threadIdx.x == 0) report_timeout(p.err);
            break;
        }
        C *buf = ring + size_t(s) * 2 * CH;
        if (split) {
            for (uint32_t q = threadIdx.x; q < CH; q += kBulkThreads) {
                C a0 = buf[q], a1 = buf[CH + q];
                body1_sel<T, BODY, EMU>(m, kc, a0, a1);
                buf[q] = a0;
                buf[CH + q] = a1;
            }
        } else {
            const uint32_t lo = (1u << p.t) - 1;
            for (uint32_t q = threadIdx.x; q < CH; q += kBulkThreads) {
                const uint32_t e0 = ((q & ~lo) << 1) | (q & lo), e1 = e0 | (1u << p.t);
                C a0 = buf[e0], a1 = buf[e1];
                body1_sel<T, BODY, EMU>(m, kc, a0, a1);
                buf[e0] = a0;
                buf[e1] = a1;
            }
        }
        fence_async_shared();
        __syncthreads();
        if (threadIdx.x == 0) {
            issue_store(tile, s);
            if (j >= 1) {
                // refill the previous stage once its store has finished reading it
                const uint64_t jp = j - 1;
                const uint64_t next = blockIdx.x + (jp + kBulkStages) * G;
                if (next < p.ntiles) {
                    bulk_wait_read1();
                    issue_load(next, int(jp % kBulkStages));
                }
            }
        }
    }
    if (failed && threadIdx.x == 0) {
        // Loads issued before the time-out may still be landing in this CTA's
        // shared memory: wait (bounded again) for each of them before leaving.
        // At iteration j the loads of iterations j .. max(2, j + 1) are out.
        const uint64_t last = j + 1 > uint64_t(kBulkStages - 1) ? j + 1 : uint64_t(kBulkStages - 1);
        for (uint64_t jj = j; jj <= last && blockIdx.x + jj * G < p.ntiles; jj++) {
            const int s = int(jj % kBulkStages);
            const uint32_t parity = uint32_t((jj / kBulkStages) & 1);
            for (uint32_t spins = 0; !mbar_try_wait(&full_bar[s], parity) && spins <= kWaitLimit; spins++) {
            }
        }
    }
    if (threadIdx.x == 0) bulk_wait_all();
}

}  // namespace lgpu

#include "lgpu_tc.cuh"

namespace lgpu {

template <class T, class I> struct PhaseParams {
    Holes holes;
    I set;  // bits forced to 1
    I ngroups;
    T re, im;
    KConst k[2];  // {-im, im} for the complex128 EMU variant
};

template <class T, class I, bool NEG, int ITEMS, bool EMU>
__global__ void __launch_bounds__(kGateBlock)
    phase_kernel(cplx_t<T> *__restrict__ sv, const PhaseParams<T, I> p, const unsigned nstates,
                 cplx_t<T> *const *__restrict__ svs) {
    using C = cplx_t<T>;
    C *s = nstates ? svs[blockIdx.y] : sv;
    const I stride = I(gridDim.x) * kGateBlock;
    for (I g = I(blockIdx.x) * kGateBlock + threadIdx.x; g < p.ngroups; g += stride * ITEMS) {
        C a[ITEMS];
        I idx[ITEMS];
#pragma unroll
        for (int k = 0; k < ITEMS; k++) {
            const I gk = g + I(k) * stride;
            idx[k] = (gk < p.ngroups) ? (insert_holes<I>(gk, p.holes) | p.set) : I(0);
            if (gk < p.ngroups) a[k] = __ldcs(&s[idx[k]]);
        }
#pragma unroll
        for (int k = 0; k < ITEMS; k++) {
            const C x = a[k];
            if constexpr (NEG) {
                a[k] = mk<T>(-x.x, -x.y);
            } else if constexpr (EMU && sizeof(T) == 8) {
                const double xr = double(x.x), xi = double(x.y), pr = double(p.re);
                a[k] = mk<T>(T(__fma_rn(pr, xr, emul(xi, p.k[0]))), T(__fma_rn(pr, xi, emul(xr, p.k[1]))));
            } else {
                a[k] = mk<T>(fmaT(p.re, x.x, -p.im * x.y), fmaT(p.re, x.y, p.im * x.x));
            }
        }
#pragma unroll
        for (int k = 0; k < ITEMS; k++)
            if (g + I(k) * stride < p.ngroups) __stcs(&s[idx[k]], a[k]);
    }
}

// Dense t-target gate, matrix in the parameter bank.
template <class T, class I, int TT> struct GkParams {
    Holes holes;
    I cset;
    I ngroups;
    I off[1 << TT];
    T m[2 * (1 << TT) * (1 << TT)];  // state precision: no conversions in the loop
};

template <class T, class I, int TT>
__global__ void __launch_bounds__(TT >= 4 ? 128 : kGateBlock)
    gatek_kernel(cplx_t<T> *__restrict__ sv, const GkParams<T, I, TT> p, const unsigned nstates,
                 cplx_t<T> *const *__restrict__ svs) {
    using C = cplx_t<T>;
    constexpr int D = 1 << TT;
    C *s = nstates ? svs[blockIdx.y] : sv;
    const I stride = I(gridDim.x) * blockDim.x;
    for (I g = I(blockIdx.x) * blockDim.x + threadIdx.x; g < p.ngroups; g += stride) {
        const I base = insert_holes<I>(g, p.holes) | p.cset;
        C a[D];
#pragma unroll
        for (int c = 0; c < D; c++) a[c] = s[base | p.off[c]];
#pragma unroll 1
        for (int r = 0; r < D; r++) {
            T xr = 0, xi = 0;
#pragma unroll
            for (int c = 0; c < D; c++) {
                const T mr = p.m[2 * (r * D + c)], mi = p.m[2 * (r * D + c) + 1];
                xr = fmaT(mr, a[c].x, xr);
                xr = fmaT(-mi, a[c].y, xr);
                xi = fmaT(mr, a[c].y, xi);
                xi = fmaT(mi, a[c].x, xi);
            }
            s[base | p.off[r]] = mk<T>(xr, xi);
        }
    }
}

// Dense t-target gate, t = 6..12, matrix (state dtype) in global memory.
// Each CTA stages GPB groups of D amplitudes in shared memory; thread j of the
// CTA produces rows j, j+blockDim, ... of every staged group.
template <class T, class I> struct GbigParams {
    Holes holes;
    I cset;
    I ngroups;
    int t;
    int batch;             // groups per CTA iteration: batch * 2^t = 4096 (or all groups)
    const I *off;          // D offsets (device)
    const cplx_t<T> *matT; // D x D, transposed: matT[c * D + r] = M[r][c] (device)
};

// Dense gates on 6..12 targets: each CTA iteration stages `batch` groups
// (4096 amplitudes) in shared memory; thread j computes rows r = j mod RB
// (+ RB, ...) of groups j / RB (+ GB, ...), RB = min(D, 256), GB = 256 / RB:
// 16 outputs per thread, each matrix element read once (coalesced, from the
// transposed copy) and used for all of the thread's groups.  State-precision
// arithmetic (FP32 for complex64, FP64 for complex128).
constexpr int kGbigThreads = 256;
constexpr int kGbigOut = 16;  // outputs per thread per iteration

template <class T, class I>
__global__ void __launch_bounds__(kGbigThreads) gatebig_kernel(cplx_t<T> *__restrict__ sv, const GbigParams<T, I> p) {
    using C = cplx_t<T>;
    extern __shared__ unsigned char smem_raw[];
    C *tile = reinterpret_cast<C *>(smem_raw);  // [batch][D]
    const int D = 1 << p.t;
    const int RB = D < kGbigThreads ? D : kGbigThreads, GB = kGbigThreads / RB;
    const int r0 = threadIdx.x % RB, gl = threadIdx.x / RB;
    const int rows = D / RB, grp = (p.batch + GB - 1) / GB;  // rows * grp <= kGbigOut
    const I nbatches = (p.ngroups + I(p.batch) - 1) / I(p.batch);
    for (I bt = blockIdx.x; bt < nbatches; bt += gridDim.x) {
        const I g0 = bt * I(p.batch);
        __syncthreads();
        for (int e = threadIdx.x; e < p.batch * D; e += kGbigThreads) {
            const int b = e / D, c = e % D;
            const I g = g0 + I(b);
            if (g < p.ngroups) tile[e] = sv[(insert_holes<I>(g, p.holes) | p.cset) | p.off[c]];
        }
        __syncthreads();
        for (int ri = 0; ri < rows; ri++) {
            const int r = r0 + ri * RB;
            C acc[kGbigOut];
#pragma unroll
            for (int q = 0; q < kGbigOut; q++) acc[q] = mk<T>(T(0), T(0));
            for (int c = 0; c < D; c++) {
                const C mv = p.matT[size_t(c) * D + r];
#pragma unroll
                for (int q = 0; q < kGbigOut; q++) {
                    if (q < grp && gl + q * GB < p.batch) {
                        const C av = tile[(gl + q * GB) * D + c];
                        acc[q] = cfma<T>(mv, av, acc[q]);
                    }
                }
            }
#pragma unroll
            for (int q = 0; q < kGbigOut; q++) {
                if (q < grp && gl + q * GB < p.batch) {
                    const I g = g0 + I(gl + q * GB);
                    if (g < p.ngroups) sv[(insert_holes<I>(g, p.holes) | p.cset) | p.off[r]] = acc[q];
                }
            }
        }
    }
}

// exp(i angle P): pairs (i, j = i ^ flip) with i's lowest flip bit clear.
template <class T, class I> struct PRParams {
    Holes holes;
    I cset;
    I ngroups;
    I flip;
    I sgn;
    T c, s;     // cos(angle), sin(angle)
    T qr, qi;   // q = s * i^(ny+1)
};

template <class T, class I>
__global__ void __launch_bounds__(kGateBlock)
    pauli_rot_kernel(cplx_t<T> *__restrict__ sv, const PRParams<T, I> p, const unsigned nstates,
                     cplx_t<T> *const *__restrict__ svs) {
    using C = cplx_t<T>;
    C *s = nstates ? svs[blockIdx.y] : sv;
    const I stride = I(gridDim.x) * kGateBlock;
    for (I g = I(blockIdx.x) * kGateBlock + threadIdx.x; g < p.ngroups; g += stride) {
        const I i = insert_holes<I>(g, p.holes) | p.cset;
        if (p.flip == 0) {
            const C a = s[i];
            const T sg = (__popcll(uint64_t(i & p.sgn)) & 1) ? T(-1) : T(1);
            const T si = p.s * sg;  // (c + i s sg) a
            s[i] = mk<T>(fmaT(p.c, a.x, -si * a.y), fmaT(p.c, a.y, si * a.x));
        } else {
            const I j = i ^ p.flip;
            const C a = s[i], b = s[j];
            const T sj = (__popcll(uint64_t(j & p.sgn)) & 1) ? T(-1) : T(1);
            const T si = (__popcll(uint64_t(i & p.sgn)) & 1) ? T(-1) : T(1);
            // out_i = c a + sj q b ; out_j = c b + si q a
            const T qbr = sj * (p.qr * b.x - p.qi * b.y), qbi = sj * (p.qr * b.y + p.qi * b.x);
            const T qar = si * (p.qr * a.x - p.qi * a.y), qai = si * (p.qr * a.y + p.qi * a.x);
            s[i] = mk<T>(fmaT(p.c, a.x, qbr), fmaT(p.c, a.y, qbi));
            s[j] = mk<T>(fmaT(p.c, b.x, qar), fmaT(p.c, b.y, qai));
        }
    }
}

// ---------------------------------------------------------------------------
// Fused shared-memory tiles
// ---------------------------------------------------------------------------
template <class T, class I> struct FusedParams {
    Holes holes;       // tile bits (sorted) as holes: tile base = insert(tau)
    I ntiles;
    int k;             // tile bits
    int m;             // low bits 0..m-1 are the lowest tile bits (contiguous runs)
    I hi_off[256];     // offsets of the high tile bits (k - m <= 8 -> 256 entries)
    int ngates;
    int ngroups;
    FGate gates[kFusedMaxGates];
    FGroup groups[kFusedMaxGates];
    T mats[kFusedMatPool];
    KConst kc[kFusedMaxGates][4];  // integer-pipe multipliers (complex128 structured bodies)
    int in_ff, out_ff;             // float-float path: the state arrives / is left in float-float form
};

// Folded diagonal gates of float-float blocks (fold_diagonal_gates in
// lgpu_fused_plan.h): the table is staged in shared memory after the tile.
constexpr size_t kDiagTableBytes = size_t(16) << kDiagTableBits;

// Amplitudes per thread in a register group: 16 (complex64).  complex128
// blocks run gate by gate: they are bound by the FP64 pipe, and the register
// footprint of a group would halve the resident CTAs.
template <class T> __host__ __device__ constexpr int fused_reg_bits() { return sizeof(T) == 4 ? 4 : 1; }

template <class T, int BODY, bool EMU, int NT>
__device__ __forceinline__ void tile_pairs(cplx_t<T> *tile, int E, int q, uint32_t in_mask, uint32_t in_val,
                                           const T *m, const KConst *k) {
    using C = cplx_t<T>;
    const uint32_t holes = in_mask | (1u << q);
    const int nfree = E >> __popc(holes);
    T mr[8];
#pragma unroll
    for (int i = 0; i < 8; i++) mr[i] = m[i];
    KConst kr[4];
#pragma unroll
    for (int i = 0; i < 4; i++) kr[i] = EMU ? k[i] : KConst{};
    PairWalk w(holes, threadIdx.x, NT);
#pragma unroll 2
    for (int f = threadIdx.x; f < nfree; f += NT) {
        const int e0 = int(w.x | in_val);
        const int e1 = e0 | (1 << q);
        w.step();
        C a0 = tile[swz<T>(e0)], a1 = tile[swz<T>(e1)];
        body1_sel<T, BODY, EMU>(mr, kr, a0, a1);
        tile[swz<T>(e0)] = a0;
        tile[swz<T>(e1)] = a1;
    }
}

// complex128 gates on a tile held in float-float form: each amplitude is a
// float4 (re.hi, im.hi, re.lo, im.lo) in the slot of its double2, so the
// layout and the swizzle are those of the complex128 tile.  The bodies run as
// paired float-float lanes (re, im) (lgpu_df2.cuh): the same operations as
// the scalar bodies in half the FP32 instructions.
template <int BODY, int NT>
__device__ __forceinline__ void tile_pairs_df(float4 *tile, int E, int q, uint32_t in_mask, uint32_t in_val,
                                              const DF *m) {
    const uint32_t holes = in_mask | (1u << q);
    const int nfree = E >> __popc(holes);
    DF2 c[8];
    if constexpr (BODY != kDfSignDiag && BODY != 2) df2_coeffs(m, c);
    const float s0 = m[0].hi, s1 = m[6].hi;  // diag(+-1, +-1): exact sign flips
    PairWalk w(holes, threadIdx.x, NT);
#pragma unroll 2
    for (int f = threadIdx.x; f < nfree; f += NT) {
        const int e0 = int(w.x | in_val);
        const int e1 = e0 | (1 << q);
        w.step();
        float4 a = tile[swz<double>(e0)], b = tile[swz<double>(e1)];
        if constexpr (BODY == kDfSignDiag) {
            a = make_float4(a.x * s0, a.y * s0, a.z * s0, a.w * s0);
            b = make_float4(b.x * s1, b.y * s1, b.z * s1, b.w * s1);
        } else if constexpr (BODY == 2) {
            const float4 t = a;
            a = b;
            b = t;
        } else {
            DF2 x{f2_pack(a.x, a.y), f2_pack(a.z, a.w)}, y{f2_pack(b.x, b.y), f2_pack(b.z, b.w)};
            body1_df2<BODY>(c, x, y);
            a = make_float4(f2_x(x.hi), f2_y(x.hi), f2_x(x.lo), f2_y(x.lo));
            b = make_float4(f2_x(y.hi), f2_y(y.hi), f2_x(y.lo), f2_y(y.lo));
        }
        tile[swz<double>(e0)] = a;
        tile[swz<double>(e1)] = b;
    }
}

// A folded diagonal (fold_diagonal_gates): every amplitude e times the phase
// table[pext(e, mask)], the table (16 float-float complex entries, staged in
// shared memory by the caller) indexed by the tile positions in `mask` in
// ascending order.
template <int NT>
__device__ __forceinline__ void tile_diag_table_df(float4 *tile, int E, uint32_t mask, const float4 *tab) {
    // index bit b = tile bit q_b (ascending): (e >> (q_b - b)) & (1 << b); a
    // missing bit shifts by 31 - b >= 28, past every bit of a tile index
    int sh[kDiagTableBits];
    {
        uint32_t mm = mask;
#pragma unroll
        for (int b = 0; b < kDiagTableBits; b++) {
            sh[b] = mm ? (__ffs(int(mm)) - 1 - b) : (31 - b);
            mm &= mm - 1u;
        }
    }
    for (int e = threadIdx.x; e < E; e += NT) {
        int idx = 0;
#pragma unroll
        for (int b = 0; b < kDiagTableBits; b++) idx |= (e >> sh[b]) & (1 << b);
        const float4 t = tab[idx];  // (re.hi, re.lo, im.hi, im.lo)
        float4 &a = tile[swz<double>(e)];
        const DF2 x{f2_pack(a.x, a.y), f2_pack(a.z, a.w)}, xs{f2_pack(a.y, a.x), f2_pack(a.w, a.z)};
        const DF2 c1{f2_pack(t.x, t.x), f2_pack(t.y, t.y)}, c2{f2_pack(-t.z, t.z), f2_pack(-t.w, t.w)};
        const DF2 y = df2_sum<2>({df2_mul(c1, x), df2_mul(c2, xs)});
        a = make_float4(f2_x(y.hi), f2_y(y.hi), f2_x(y.lo), f2_y(y.lo));
    }
}

// Dense 4x4 (2-target) gate on a float-float tile; qa = most significant
// matrix bit.
template <int NT>
__device__ __forceinline__ void tile_quads_df(float4 *tile, int E, int qa, int qb, uint32_t in_mask, uint32_t in_val,
                                              const DF *m) {
    const uint32_t holes = in_mask | (1u << qa) | (1u << qb);
    const int nfree = E >> __popc(holes);
    PairWalk w(holes, threadIdx.x, NT);
    for (int f = threadIdx.x; f < nfree; f += NT) {
        const int e = int(w.x | in_val);
        w.step();
        int idx[4];
        idx[0] = swz<double>(e);
        idx[1] = swz<double>(e | (1 << qb));
        idx[2] = swz<double>(e | (1 << qa));
        idx[3] = swz<double>(e | (1 << qa) | (1 << qb));
        DF ar[4], ai[4];
#pragma unroll
        for (int c = 0; c < 4; c++) {
            const float4 v = tile[idx[c]];  // (re.hi, im.hi, re.lo, im.lo)
            ar[c] = DF{v.x, v.z};
            ai[c] = DF{v.y, v.w};
        }
#pragma unroll
        for (int r = 0; r < 4; r++) {
            DF tr[8], ti[8];
#pragma unroll
            for (int c = 0; c < 4; c++) {
                const DF mre = m[2 * (r * 4 + c)], mim = m[2 * (r * 4 + c) + 1];
                tr[2 * c] = df_mul(mre, ar[c]);
                tr[2 * c + 1] = df_mul(df_neg(mim), ai[c]);
                ti[2 * c] = df_mul(mre, ai[c]);
                ti[2 * c + 1] = df_mul(mim, ar[c]);
            }
            const DF xr = df_sum<8>(tr), xi = df_sum<8>(ti);
            tile[idx[r]] = make_float4(xr.hi, xi.hi, xr.lo, xi.lo);
        }
    }
}

// All gates of a launch on one tile held in shared memory (all threads; the
// caller synchronises before and after).  DFM (complex128): the tile holds
// float-float amplitudes (converted after the load and at the store, unless
// the state already arrives / stays in float-float form: in_ff / out_ff) and
// every gate runs in float-float arithmetic, its coefficients stored as
// (hi, lo) float pairs in the double slots of the matrix pool.
template <class T, class I, bool EMU, int NT, bool DFM = false>
__device__ __forceinline__ void fused_tile(cplx_t<T> *tile, int E, I base, const FusedParams<T, I> &p) {
    using C = cplx_t<T>;
    constexpr int R = fused_reg_bits<T>();
    for (int gr = 0; gr < p.ngroups; gr++) {
        const FGroup &G = p.groups[gr];
        if constexpr (sizeof(T) == 4) {
            if (G.kind == 0) {
                uint32_t M = 0;
#pragma unroll
                for (int b = 0; b < R; b++) M |= 1u << G.p[b];
                // swz is XOR-linear and the slot base and the offsets have
                // disjoint bits: swz(b0 | off) = swz(b0) ^ swz(off)
                int soff[1 << R];
#pragma unroll
                for (int j = 0; j < (1 << R); j++) {
                    int o = 0;
#pragma unroll
                    for (int b = 0; b < R; b++)
                        if ((j >> b) & 1) o |= 1 << G.p[b];
                    soff[j] = swz<T>(o);
                }
                const int nslots = E >> R;
                PairWalk w(M, threadIdx.x, NT);
                for (int f = threadIdx.x; f < nslots; f += NT) {
                    const int sb = swz<T>(int(w.x));
                    w.step();
                    C a[1 << R];
#pragma unroll
                    for (int j = 0; j < (1 << R); j++) a[j] = tile[sb ^ soff[j]];
                    for (int gi = G.first; gi < G.first + G.count; gi++) {
                        const FGate &g = p.gates[gi];
                        if ((uint64_t(base) & g.out_mask) != g.out_val) continue;  // tile-uniform
                        reg_gate_any<T, R, EMU>(a, g.body, g.lt, p.mats + g.mat_off, p.kc[gi], g.lcm, g.lcv);
                    }
#pragma unroll
                    for (int j = 0; j < (1 << R); j++) tile[sb ^ soff[j]] = a[j];
                }
                __syncthreads();
                continue;
            }
        }
        // complex128 launches hold one group per gate, in gate order
        const int gi = sizeof(T) == 4 ? int(G.first) : gr;
        const FGate &g = p.gates[gi];
        if ((uint64_t(base) & g.out_mask) != g.out_val) continue;  // tile-uniform
        const T *mm = p.mats + g.mat_off;
        if constexpr (DFM && sizeof(T) == 8) {
            float4 *t4 = reinterpret_cast<float4 *>(tile);
            const DF *md = reinterpret_cast<const DF *>(mm);
            if (g.ntgt == kDiagTableMark) {
                // stage the table after the tile (float-float launches are single-buffered)
                float4 *tab = reinterpret_cast<float4 *>(t4 + E);
                if (threadIdx.x < (1 << kDiagTableBits))
                    tab[threadIdx.x] = reinterpret_cast<const float4 *>(md)[threadIdx.x];
                __syncthreads();
                tile_diag_table_df<NT>(t4, E, g.in_mask, tab);
            } else if (g.ntgt == 1) {
                switch (g.pad == 1 ? kDfSignDiag : int(g.body)) {
                case kDfSignDiag: tile_pairs_df<kDfSignDiag, NT>(t4, E, g.q0, g.in_mask, g.in_val, md); break;
                case B_DIAG: tile_pairs_df<B_DIAG, NT>(t4, E, g.q0, g.in_mask, g.in_val, md); break;
                case B_PERM: tile_pairs_df<B_PERM, NT>(t4, E, g.q0, g.in_mask, g.in_val, md); break;
                case B_ANTIDIAG: tile_pairs_df<B_ANTIDIAG, NT>(t4, E, g.q0, g.in_mask, g.in_val, md); break;
                case B_REAL: tile_pairs_df<B_REAL, NT>(t4, E, g.q0, g.in_mask, g.in_val, md); break;
                case B_RXLIKE: tile_pairs_df<B_RXLIKE, NT>(t4, E, g.q0, g.in_mask, g.in_val, md); break;
                default: tile_pairs_df<B_DENSE, NT>(t4, E, g.q0, g.in_mask, g.in_val, md); break;
                }
            } else {
                tile_quads_df<NT>(t4, E, g.q0, g.q1, g.in_mask, g.in_val, md);
            }
        } else if (g.ntgt == 1) {
            const KConst *kk = p.kc[gi];
            switch (g.body) {
            case B_DIAG: tile_pairs<T, B_DIAG, EMU, NT>(tile, E, g.q0, g.in_mask, g.in_val, mm, kk); break;
            case B_PERM: tile_pairs<T, B_PERM, EMU, NT>(tile, E, g.q0, g.in_mask, g.in_val, mm, kk); break;
            case B_ANTIDIAG: tile_pairs<T, B_ANTIDIAG, EMU, NT>(tile, E, g.q0, g.in_mask, g.in_val, mm, kk); break;
            case B_REAL: tile_pairs<T, B_REAL, EMU, NT>(tile, E, g.q0, g.in_mask, g.in_val, mm, kk); break;
            case B_RXLIKE: tile_pairs<T, B_RXLIKE, EMU, NT>(tile, E, g.q0, g.in_mask, g.in_val, mm, kk); break;
            default: tile_pairs<T, B_DENSE, EMU, NT>(tile, E, g.q0, g.in_mask, g.in_val, mm, kk); break;
            }
        } else {
            const int qa = g.q0, qb = g.q1;  // qa = most significant matrix bit
            const uint32_t holes = g.in_mask | (1u << qa) | (1u << qb);
            const int nfree = E >> __popc(holes);
            PairWalk w(holes, threadIdx.x, NT);
            for (int f = threadIdx.x; f < nfree; f += NT) {
                const int e = int(w.x | g.in_val);
                w.step();
                int idx[4];
                idx[0] = swz<T>(e);
                idx[1] = swz<T>(e | (1 << qb));
                idx[2] = swz<T>(e | (1 << qa));
                idx[3] = swz<T>(e | (1 << qa) | (1 << qb));
                C a[4];
#pragma unroll
                for (int c = 0; c < 4; c++) a[c] = tile[idx[c]];
#pragma unroll
                for (int r = 0; r < 4; r++) {
                    T xr = 0, xi = 0;
#pragma unroll
                    for (int c = 0; c < 4; c++) {
                        const T mr = mm[2 * (r * 4 + c)], mi = mm[2 * (r * 4 + c) + 1];
                        xr = fmaT(mr, a[c].x, fmaT(-mi, a[c].y, xr));
                        xi = fmaT(mr, a[c].y, fmaT(mi, a[c].x, xi));
                    }
                    tile[idx[r]] = mk<T>(xr, xi);
                }
            }
        }
        __syncthreads();
    }
}

__device__ __forceinline__ void cp_async16(void *smem_dst, const void *gsrc) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(static_cast<uint32_t>(__cvta_generic_to_shared(smem_dst))),
                 "l"(gsrc)
                 : "memory");
}
__device__ __forceinline__ void cp_async8(void *smem_dst, const void *gsrc) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(static_cast<uint32_t>(__cvta_generic_to_shared(smem_dst))),
                 "l"(gsrc)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait1() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait0() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

// Persistent CTAs with a ring of STAGES tile buffers: while the gates run on
// one tile, the next STAGES - 1 tiles stream in through cp.async (16-byte
// chunks written straight into the swizzled layout); results leave with
// streaming stores.  STAGES = 1 loads and computes in turn (several CTAs per
// SM interleave instead).  The tile = the low run of m state bits (contiguous
// segments of 2^m amplitudes) times up to 2^6 segments at the high tile bits.
template <int N> __device__ __forceinline__ void cp_async_wait_n() {
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

template <class T, class I, bool EMU, int NT, int STAGES, int MINB, bool DFM = false>
__global__ void __launch_bounds__(NT, MINB)
    fused_kernel(cplx_t<T> *__restrict__ sv, const FusedParams<T, I> p) {
    static_assert(!DFM || STAGES == 1, "float-float blocks are single-buffered: the phase table follows the tile");
    using C = cplx_t<T>;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const int E = 1 << p.k;
    C *const ring = reinterpret_cast<C *>(smem_raw);
    const int lowmask = (1 << p.m) - 1;
    // 16-byte chunks hold 2 complex64 / 1 complex128 amplitudes; complex64
    // needs an even low run (always, except for a tile without bit 0)
    constexpr int EPC = sizeof(C) == 8 ? 2 : 1;
    const bool wide = EPC == 1 || p.m >= 1;
    auto load = [&](I tau, C *dst) {
        const I base = insert_holes<I>(tau, p.holes);
        if (wide) {
            for (int c = threadIdx.x; c < E / EPC; c += NT) {
                const int e = c * EPC;
                cp_async16(&dst[swz<T>(e)], &sv[base + p.hi_off[e >> p.m] + I(e & lowmask)]);
            }
        } else {
            for (int e = threadIdx.x; e < E; e += NT)
                cp_async8(&dst[swz<T>(e)], &sv[base + p.hi_off[e >> p.m] + I(e & lowmask)]);
        }
        cp_async_commit();
    };
    const I G = I(gridDim.x);
    if constexpr (STAGES > 1) {
#pragma unroll
        for (int s = 0; s < STAGES - 1; s++) {
            const I t = I(blockIdx.x) + I(s) * G;
            if (t < p.ntiles) load(t, ring + size_t(s) * E);
            else cp_async_commit();
        }
    }
    int it = 0;
    for (I tau = blockIdx.x; tau < p.ntiles; tau += G, it++) {
        C *cur = ring + size_t(STAGES > 1 ? it % STAGES : 0) * E;
        if constexpr (STAGES > 1) {
            // the buffer of iteration it - 1, freed by its closing barrier
            const I tn = tau + I(STAGES - 1) * G;
            if (tn < p.ntiles) load(tn, ring + size_t((it + STAGES - 1) % STAGES) * E);
            else cp_async_commit();
            cp_async_wait_n<STAGES - 1>();  // this thread's copies of `cur` have landed
        } else {
            load(tau, cur);
            cp_async_wait0();
        }
        __syncthreads();  // ... and everyone's
        if constexpr (DFM && sizeof(T) == 8) {
            if (!p.in_ff) {  // complex128 -> float-float in place (same 16 bytes per amplitude)
                for (int e = threadIdx.x; e < E; e += NT) {
                    const double2 v = reinterpret_cast<const double2 *>(cur)[e];
                    const DF r = df_from_double(v.x), i = df_from_double(v.y);
                    reinterpret_cast<float4 *>(cur)[e] = make_float4(r.hi, i.hi, r.lo, i.lo);
                }
                __syncthreads();
            }
        }
        const I base = insert_holes<I>(tau, p.holes);
        fused_tile<T, I, EMU, NT, DFM>(cur, E, base, p);
        if (wide) {
            for (int c = threadIdx.x; c < E / EPC; c += NT) {
                const int e = c * EPC;
                C *dst = &sv[base + p.hi_off[e >> p.m] + I(e & lowmask)];
                if constexpr (EPC == 2) {
                    __stcs(reinterpret_cast<float4 *>(dst), *reinterpret_cast<const float4 *>(&cur[swz<T>(e)]));
                } else if constexpr (DFM && sizeof(T) == 8) {
                    const float4 v = reinterpret_cast<const float4 *>(cur)[swz<T>(e)];
                    if (p.out_ff)
                        __stcs(reinterpret_cast<float4 *>(dst), v);
                    else
                        __stcs(reinterpret_cast<double2 *>(dst),
                               make_double2(df_to_double(DF{v.x, v.z}), df_to_double(DF{v.y, v.w})));
                } else {
                    __stcs(dst, cur[swz<T>(e)]);
                }
            }
        } else {
            for (int e = threadIdx.x; e < E; e += NT)
                __stcs(&sv[base + p.hi_off[e >> p.m] + I(e & lowmask)], cur[swz<T>(e)]);
        }
        __syncthreads();  // `cur` is the target of a load issued next iteration
    }
    cp_async_wait0();
}

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
struct Cm {
    double re, im;
};
static inline bool eq(Cm a, double re, double im) { return a.re == re && a.im == im; }

struct GateGeometry {
    std::vector<int> tgts, ctrls, cvals;
    uint64_t cset = 0;
};

static lgpu_status_t geometry(uint32_t n, uint32_t t, const int32_t *tgts, uint32_t c,
                              const int32_t *ctrls, const int32_t *ctrl_vals, GateGeometry *g) {
    if (t < 1 || t > LGPU_MAX_DENSE_TARGETS)
        return fail(LGPU_ERR_INVALID_ARG, "number of targets must be in [1, 12]");
    if (c > LGPU_MAX_CONTROLS) return fail(LGPU_ERR_INVALID_ARG, "too many controls");
    LGPU_TRY(check_bits(n, t, tgts, "target", &g->tgts));
    LGPU_TRY(check_bits(n, c, ctrls, "control", &g->ctrls));
    std::vector<int> all(g->tgts);
    all.insert(all.end(), g->ctrls.begin(), g->ctrls.end());
    std::vector<int> srt(all);
    std::sort(srt.begin(), srt.end());
    if (std::adjacent_find(srt.begin(), srt.end()) != srt.end())
        return fail(LGPU_ERR_INVALID_ARG, "target and control bits must be distinct");
    if (all.size() > n) return fail(LGPU_ERR_INVALID_ARG, "more wires than qubits");
    for (uint32_t k = 0; k < c; k++) {
        const int v = ctrl_vals ? ctrl_vals[k] : 1;
        if (v != 0 && v != 1) return fail(LGPU_ERR_INVALID_ARG, "control values must be 0 or 1");
        g->cvals.push_back(v);
        if (v) g->cset |= uint64_t(1) << g->ctrls[k];
    }
    return LGPU_OK;
}

template <class T, class I, int BODY>
static void launch_gate1(cplx_t<T> *sv, const G1Params<T, I> &p, unsigned nstates,
                         cplx_t<T> *const *svs, cudaStream_t s) {
    constexpr int ITEMS = sizeof(T) == 8 ? 2 : 4;
    const unsigned gx = grid_for(uint64_t(p.ngroups), kGateBlock, ITEMS, 8);
    dim3 grid(gx, nstates ? nstates : 1);
    if constexpr (sizeof(T) == 8) {
        if (f64_mode() == 1) {
            gate1_kernel<T, I, BODY, ITEMS, true><<<grid, kGateBlock, 0, s>>>(sv, p, nstates, svs);
            return;
        }
    }
    gate1_kernel<T, I, BODY, ITEMS, false><<<grid, kGateBlock, 0, s>>>(sv, p, nstates, svs);
}

template <class T, int BODY, bool EMU>
static lgpu_status_t launch_bulk_t(cplx_t<T> *sv, const BulkParams<T> &bp, cudaStream_t s) {
    const size_t smem = size_t(kBulkStages) * (size_t(2) << bp.ch_log2) * sizeof(cplx_t<T>);
    static std::atomic<size_t> attr[64];
    LGPU_TRY(ensure_smem(reinterpret_cast<const void *>(gate1_bulk_kernel<T, BODY, EMU>), smem, attr));
    const unsigned grid = unsigned(std::min<uint64_t>(bp.ntiles, uint64_t(sm_count())));
    gate1_bulk_kernel<T, BODY, EMU><<<grid, kBulkThreads, smem, s>>>(sv, bp);
    LGPU_CHECK_LAUNCH();
    return LGPU_OK;
}

template <class T, bool EMU>
static lgpu_status_t launch_bulk_body(cplx_t<T> *sv, const BulkParams<T> &bp, int body, cudaStream_t s) {
    switch (body) {
    case B_DIAG: return launch_bulk_t<T, B_DIAG, EMU>(sv, bp, s);
    case B_PERM: return launch_bulk_t<T, B_PERM, false>(sv, bp, s);
    case B_ANTIDIAG: return launch_bulk_t<T, B_ANTIDIAG, EMU>(sv, bp, s);
    case B_REAL: return launch_bulk_t<T, B_REAL, EMU>(sv, bp, s);
    case B_RXLIKE: return launch_bulk_t<T, B_RXLIKE, EMU>(sv, bp, s);
    default: return launch_bulk_t<T, B_DENSE, EMU>(sv, bp, s);
    }
}

template <class T>
static lgpu_status_t launch_gate1_bulk(cplx_t<T> *sv, const BulkParams<T> &bp, int body, cudaStream_t s) {
    if constexpr (sizeof(T) == 8) {
        if (f64_mode() == 1) return launch_bulk_body<T, true>(sv, bp, body, s);
    }
    return launch_bulk_body<T, false>(sv, bp, body, s);
}

template <class T, class I>
static lgpu_status_t run_gate1(cplx_t<T> *sv, unsigned nstates, cplx_t<T> *const *svs, uint32_t n,
                               const Cm m[4], const GateGeometry &g, cudaStream_t s) {
    const int tb = g.tgts[0];
    // Phase-only gates touch the amplitudes of one target value only.
    const bool diag = eq(m[1], 0, 0) && eq(m[2], 0, 0);
    if (diag && (eq(m[0], 1, 0) || eq(m[3], 1, 0))) {
        const bool on_one = eq(m[0], 1, 0);
        const Cm ph = on_one ? m[3] : m[0];
        if (eq(ph, 1, 0)) return LGPU_OK;  // identity
        std::vector<int> holes(g.ctrls);
        holes.push_back(tb);
        PhaseParams<T, I> p{};
        p.holes = make_holes(holes);
        p.set = I(g.cset | (on_one ? (uint64_t(1) << tb) : 0));
        p.ngroups = I(uint64_t(1) << (n - holes.size()));
        p.re = T(ph.re);
        p.im = T(ph.im);
        p.k[0] = make_kconst(-ph.im);
        p.k[1] = make_kconst(ph.im);
        constexpr int ITEMS = sizeof(T) == 8 ? 2 : 4;
        dim3 grid(grid_for(uint64_t(p.ngroups), kGateBlock, ITEMS, 8), nstates ? nstates : 1);
        bool emu = false;
        if constexpr (sizeof(T) == 8) emu = f64_mode() == 1;
        if (eq(ph, -1, 0)) {
            phase_kernel<T, I, true, ITEMS, false><<<grid, kGateBlock, 0, s>>>(sv, p, nstates, svs);
        } else if (emu) {
            if constexpr (sizeof(T) == 8)
                phase_kernel<T, I, false, ITEMS, true><<<grid, kGateBlock, 0, s>>>(sv, p, nstates, svs);
        } else {
            phase_kernel<T, I, false, ITEMS, false><<<grid, kGateBlock, 0, s>>>(sv, p, nstates, svs);
        }
        LGPU_CHECK_LAUNCH();
        return LGPU_OK;
    }
    std::vector<int> holes(g.ctrls);
    holes.push_back(tb);
    G1Params<T, I> p{};
    p.holes = make_holes(holes);
    p.tbit = I(uint64_t(1) << tb);
    p.cset = I(g.cset);
    p.ngroups = I(uint64_t(1) << (n - holes.size()));
    for (int k = 0; k < 4; k++) {
        p.m[2 * k] = T(m[k].re);
        p.m[2 * k + 1] = T(m[k].im);
    }
    const bool anti = eq(m[0], 0, 0) && eq(m[3], 0, 0);
    const bool real = m[0].im == 0 && m[1].im == 0 && m[2].im == 0 && m[3].im == 0;
    const bool rxlike = m[0].im == 0 && m[3].im == 0 && m[0].re == m[3].re && m[1].re == 0 && m[2].re == 0;
    if (diag) {
        p.k[0] = make_kconst(-m[0].im); p.k[1] = make_kconst(m[0].im);
        p.k[2] = make_kconst(-m[3].im); p.k[3] = make_kconst(m[3].im);
    } else if (anti) {
        p.k[0] = make_kconst(-m[1].im); p.k[1] = make_kconst(m[1].im);
        p.k[2] = make_kconst(-m[2].im); p.k[3] = make_kconst(m[2].im);
    } else if (real) {
        p.k[0] = make_kconst(m[1].re); p.k[1] = make_kconst(m[2].re);
    } else if (rxlike) {
        p.k[0] = make_kconst(-m[1].im); p.k[1] = make_kconst(m[1].im);
        p.k[2] = make_kconst(-m[2].im); p.k[3] = make_kconst(m[2].im);
    } else {  // dense
        p.k[0] = make_kconst(m[0].im); p.k[1] = make_kconst(m[1].im);
        p.k[2] = make_kconst(m[2].im); p.k[3] = make_kconst(m[3].im);
    }
    if (nstates == 0 && g.ctrls.empty() && bulk_enabled()) {
        const int ch_log2 = sizeof(T) == 8 ? 11 : 12;  // 32 KB halves, 64 KB tiles
        if (int(n) >= ch_log2 + 2) {
            BulkParams<T> bp{};
            LGPU_TRY(stream_error_ptr(s, &bp.err));
            bp.ntiles = (uint64_t(1) << n) >> (ch_log2 + 1);
            bp.t = tb;
            bp.ch_log2 = ch_log2;
            for (int q = 0; q < 8; q++) bp.m[q] = p.m[q];
            for (int q = 0; q < 4; q++) bp.k[q] = p.k[q];
            const int body = diag ? B_DIAG : (anti && eq(m[1], 1, 0) && eq(m[2], 1, 0)) ? B_PERM : anti ? B_ANTIDIAG
                             : real ? B_REAL : rxlike ? B_RXLIKE : B_DENSE;
            return launch_gate1_bulk<T>(sv, bp, body, s);
        }
    }
    if (diag)
        launch_gate1<T, I, B_DIAG>(sv, p, nstates, svs, s);
    else if (anti && eq(m[1], 1, 0) && eq(m[2], 1, 0))
        launch_gate1<T, I, B_PERM>(sv, p, nstates, svs, s);
    else if (anti)
        launch_gate1<T, I, B_ANTIDIAG>(sv, p, nstates, svs, s);
    else if (real)
        launch_gate1<T, I, B_REAL>(sv, p, nstates, svs, s);
    else if (rxlike)
        launch_gate1<T, I, B_RXLIKE>(sv, p, nstates, svs, s);
    else
        launch_gate1<T, I, B_DENSE>(sv, p, nstates, svs, s);
    LGPU_CHECK_LAUNCH();
    return LGPU_OK;
}

template <class T, class I, int TT>
static lgpu_status_t run_gatek(cplx_t<T> *sv, unsigned nstates, cplx_t<T> *const *svs, uint32_t n,
                               const std::vector<Cm> &m, const GateGeometry &g, cudaStream_t s) {
    constexpr int D = 1 << TT;
    auto *p = new GkParams<T, I, TT>();
    std::vector<int> holes(g.ctrls);
    holes.insert(holes.end(), g.tgts.begin(), g.tgts.end());
    p->holes = make_holes(holes);
    p->cset = I(g.cset);
    p->ngroups = I(uint64_t(1) << (n - holes.size()));
    for (int r = 0; r < D; r++) {
        uint64_t o = 0;
        for (int k = 0; k < TT; k++)
            if ((r >> (TT - 1 - k)) & 1) o |= uint64_t(1) << g.tgts[size_t(k)];
        p->off[r] = I(o);
    }
    for (int e = 0; e < D * D; e++) {
        p->m[2 * e] = T(m[size_t(e)].re);
        p->m[2 * e + 1] = T(m[size_t(e)].im);
    }
    const int block = TT >= 4 ? 128 : kGateBlock;
    dim3 grid(grid_for(uint64_t(p->ngroups), block, 1, 8), nstates ? nstates : 1);
    gatek_kernel<T, I, TT><<<grid, block, 0, s>>>(sv, *p, nstates, svs);
    delete p;
    LGPU_CHECK_LAUNCH();
    return LGPU_OK;
}

template <class T, class I>
static lgpu_status_t run_gatebig(cplx_t<T> *sv, uint32_t n, const std::vector<Cm> &m,
                                 const GateGeometry &g, cudaStream_t s) {
    const int t = int(g.tgts.size());
    const int D = 1 << t;
    std::vector<I> off(static_cast<size_t>(D));
    for (int r = 0; r < D; r++) {
        uint64_t o = 0;
        for (int k = 0; k < t; k++)
            if ((r >> (t - 1 - k)) & 1) o |= uint64_t(1) << g.tgts[size_t(k)];
        off[size_t(r)] = I(o);
    }
    std::vector<cplx_t<T>> mh(size_t(D) * D);  // transposed
    for (int r = 0; r < D; r++)
        for (int c = 0; c < D; c++) {
            const Cm v = m[size_t(r) * D + c];
            mh[size_t(c) * D + r] = mk<T>(T(v.re), T(v.im));
        }
    // Stream-ordered pool allocation for the device copy of the matrix.
    void *dbuf = nullptr;
    const size_t mbytes = mh.size() * sizeof(cplx_t<T>), obytes = off.size() * sizeof(I);
    LGPU_CUDA_TRY(cudaMallocAsync(&dbuf, mbytes + obytes + 256, s));
    auto *dmat = static_cast<cplx_t<T> *>(dbuf);
    auto *doff = reinterpret_cast<I *>(static_cast<char *>(dbuf) + ((mbytes + 255) & ~size_t(255)));
    LGPU_CUDA_TRY(cudaMemcpyAsync(dmat, mh.data(), mbytes, cudaMemcpyHostToDevice, s));
    LGPU_CUDA_TRY(cudaMemcpyAsync(doff, off.data(), obytes, cudaMemcpyHostToDevice, s));
    std::vector<int> holes(g.ctrls);
    holes.insert(holes.end(), g.tgts.begin(), g.tgts.end());
    GbigParams<T, I> p{};
    p.holes = make_holes(holes);
    p.cset = I(g.cset);
    p.ngroups = I(uint64_t(1) << (n - holes.size()));
    p.t = t;
    p.batch = int(std::min<uint64_t>(uint64_t(4096 / D), uint64_t(p.ngroups)));
    if (p.batch < 1) p.batch = 1;
    p.off = doff;
    p.matT = dmat;
    const size_t smem = size_t(p.batch) * D * sizeof(cplx_t<T>);
    static std::atomic<size_t> attr[64];
    LGPU_TRY(ensure_smem(reinterpret_cast<const void *>(gatebig_kernel<T, I>), smem, attr));
    const uint64_t nbatches = (uint64_t(p.ngroups) + p.batch - 1) / p.batch;
    const unsigned per_sm = sizeof(T) == 8 ? 3 : 6;
    const unsigned grid = unsigned(std::min<uint64_t>(nbatches, uint64_t(sm_count()) * per_sm));
    gatebig_kernel<T, I><<<grid, kGbigThreads, smem, s>>>(sv, p);
    LGPU_CHECK_LAUNCH();
    LGPU_CUDA_TRY(cudaFreeAsync(dbuf, s));
    return LGPU_OK;
}

// Dense 6-target complex64 gate on the six lowest state bits (targets in any
// order, no controls) on the tensor cores: U is reordered so that row and
// column indices are the state's own low six bits.
static bool dense6_tc_applies(uint32_t n, uint32_t t, const GateGeometry &g) {
    if (t != 6 || n < 12 || !g.ctrls.empty() || !tc_enabled()) return false;
    uint32_t seen = 0;
    for (int b : g.tgts) {
        if (b < 0 || b > 5) return false;
        seen |= 1u << b;
    }
    return seen == 0x3Fu;
}

static lgpu_status_t run_dense6_tc(float2 *sv, uint32_t n, const std::vector<Cm> &m, const GateGeometry &g,
                                   cudaStream_t s) {
    int rowof[64];
    for (int x = 0; x < 64; x++) {
        int r = 0;
        for (int k = 0; k < 6; k++)
            if ((x >> g.tgts[size_t(k)]) & 1) r |= 1 << (5 - k);
        rowof[x] = r;
    }
    std::vector<float2> u(64 * 64);
    for (int x = 0; x < 64; x++)
        for (int y = 0; y < 64; y++) {
            const Cm v = m[size_t(rowof[x] * 64 + rowof[y])];
            u[size_t(x * 64 + y)] = make_float2(float(v.re), float(v.im));
        }
    void *dbuf = nullptr;
    const size_t bytes = u.size() * sizeof(float2);
    LGPU_CUDA_TRY(cudaMallocAsync(&dbuf, bytes, s));
    LGPU_CUDA_TRY(cudaMemcpyAsync(dbuf, u.data(), bytes, cudaMemcpyHostToDevice, s));
    TcDense6Params p{};
    LGPU_TRY(stream_error_ptr(s, &p.err));
    p.u = static_cast<const float2 *>(dbuf);
    p.ntiles = (uint64_t(1) << n) / uint64_t(kTcTileAmps);
    static std::atomic<size_t> attr[64];
    LGPU_TRY(ensure_smem(reinterpret_cast<const void *>(dense6_tc_kernel), kTcSmemBytes, attr));
    const unsigned grid = unsigned(std::min<uint64_t>(p.ntiles, uint64_t(sm_count())));
    dense6_tc_kernel<<<grid, kTcThreads, kTcSmemBytes, s>>>(sv, p);
    LGPU_CHECK_LAUNCH();
    LGPU_CUDA_TRY(cudaFreeAsync(dbuf, s));
    return LGPU_OK;
}

template <class T, class I>
static lgpu_status_t apply_matrix_t(cplx_t<T> *sv, unsigned nstates, cplx_t<T> *const *svs, uint32_t n,
                                    const double *matrix, uint32_t t, const GateGeometry &g,
                                    int adjoint, cudaStream_t s) {
    const int D = 1 << t;
    std::vector<Cm> m(size_t(D) * D);
    for (int r = 0; r < D; r++)
        for (int c = 0; c < D; c++) {
            const int src = adjoint ? (c * D + r) : (r * D + c);
            m[size_t(r * D + c)] = {matrix[2 * src], adjoint ? -matrix[2 * src + 1] : matrix[2 * src + 1]};
        }
    switch (t) {
    case 1: return run_gate1<T, I>(sv, nstates, svs, n, m.data(), g, s);
    case 2: return run_gatek<T, I, 2>(sv, nstates, svs, n, m, g, s);
    case 3: return run_gatek<T, I, 3>(sv, nstates, svs, n, m, g, s);
    case 4: return run_gatek<T, I, 4>(sv, nstates, svs, n, m, g, s);
    case 5: return run_gatek<T, I, 5>(sv, nstates, svs, n, m, g, s);
    default:
        // t > 5: multi-state calls are split per state by the caller
        if constexpr (sizeof(T) == 4)
            if (dense6_tc_applies(n, t, g)) return run_dense6_tc(sv, n, m, g, s);
        return run_gatebig<T, I>(sv, n, m, g, s);
    }
}

// Multi-state launches read the state pointers from a small device array held
// in stream-ordered pool memory.
template <class T>
static lgpu_status_t with_state_array(void *const *svs, uint32_t nstates, cudaStream_t s,
                                      cplx_t<T> ***dev_out, void **to_free) {
    void *buf = nullptr;
    LGPU_CUDA_TRY(cudaMallocAsync(&buf, sizeof(void *) * nstates, s));
    LGPU_CUDA_TRY(cudaMemcpyAsync(buf, svs, sizeof(void *) * nstates, cudaMemcpyHostToDevice, s));
    *dev_out = static_cast<cplx_t<T> **>(buf);
    *to_free = buf;
    return LGPU_OK;
}

template <class T>
static lgpu_status_t apply_matrix_dispatch(void *sv, void *const *svs, uint32_t nstates, uint32_t n,
                                           const double *matrix, uint32_t t, const GateGeometry &g,
                                           int adjoint, cudaStream_t s) {
    if (nstates && t > 5) {
        for (uint32_t k = 0; k < nstates; k++) {
            lgpu_status_t st = n <= 32 ? apply_matrix_t<T, uint32_t>(static_cast<cplx_t<T> *>(svs[k]), 0,
                                                                     nullptr, n, matrix, t, g, adjoint, s)
                                       : apply_matrix_t<T, uint64_t>(static_cast<cplx_t<T> *>(svs[k]), 0,
                                                                     nullptr, n, matrix, t, g, adjoint, s);
            if (st != LGPU_OK) return st;
        }
        return LGPU_OK;
    }
    cplx_t<T> **dev = nullptr;
    void *to_free = nullptr;
    if (nstates) LGPU_TRY(with_state_array<T>(svs, nstates, s, &dev, &to_free));
    lgpu_status_t st = n <= 32 ? apply_matrix_t<T, uint32_t>(static_cast<cplx_t<T> *>(sv), nstates, dev, n,
                                                             matrix, t, g, adjoint, s)
                               : apply_matrix_t<T, uint64_t>(static_cast<cplx_t<T> *>(sv), nstates, dev, n,
                                                             matrix, t, g, adjoint, s);
    if (to_free) cudaFreeAsync(to_free, s);
    return st;
}

template <class T, class I>
static lgpu_status_t pauli_rot_t(cplx_t<T> *sv, unsigned nstates, cplx_t<T> *const *svs, uint32_t n,
                                 double angle, const GateGeometry &g, const char *paulis, cudaStream_t s) {
    uint64_t flip = 0, sgn = 0;
    int ny = 0;
    for (size_t k = 0; k < g.tgts.size(); k++) {
        const uint64_t b = uint64_t(1) << g.tgts[k];
        switch (paulis[k]) {
        case 'X': flip |= b; break;
        case 'Y': flip |= b; sgn |= b; ny++; break;
        case 'Z': sgn |= b; break;
        case 'I': break;
        default: return fail(LGPU_ERR_INVALID_ARG, std::string("bad Pauli letter '") + paulis[k] + "'");
        }
    }
    PRParams<T, I> p{};
    std::vector<int> holes(g.ctrls);
    if (flip) holes.push_back(__builtin_ctzll(flip));
    p.holes = make_holes(holes);
    p.cset = I(g.cset);
    p.ngroups = I(uint64_t(1) << (n - holes.size()));
    p.flip = I(flip);
    p.sgn = I(sgn);
    p.c = T(std::cos(angle));
    p.s = T(std::sin(angle));
    // q = s * i^(ny+1)
    const double sv_ = std::sin(angle);
    switch ((ny + 1) & 3) {
    case 0: p.qr = T(sv_); p.qi = 0; break;
    case 1: p.qr = 0; p.qi = T(sv_); break;
    case 2: p.qr = T(-sv_); p.qi = 0; break;
    default: p.qr = 0; p.qi = T(-sv_); break;
    }
    dim3 grid(grid_for(uint64_t(p.ngroups), kGateBlock, 2, 8), nstates ? nstates : 1);
    pauli_rot_kernel<T, I><<<grid, kGateBlock, 0, s>>>(sv, p, nstates, svs);
    LGPU_CHECK_LAUNCH();
    return LGPU_OK;
}

template <class T>
static lgpu_status_t pauli_rot_dispatch(void *sv, void *const *svs, uint32_t nstates, uint32_t n,
                                        double angle, const GateGeometry &g, const char *paulis,
                                        cudaStream_t s) {
    cplx_t<T> **dev = nullptr;
    void *to_free = nullptr;
    if (nstates) LGPU_TRY(with_state_array<T>(svs, nstates, s, &dev, &to_free));
    lgpu_status_t st = n <= 32 ? pauli_rot_t<T, uint32_t>(static_cast<cplx_t<T> *>(sv), nstates, dev, n, angle,
                                                          g, paulis, s)
                               : pauli_rot_t<T, uint64_t>(static_cast<cplx_t<T> *>(sv), nstates, dev, n,
                                                          angle, g, paulis, s);
    if (to_free) cudaFreeAsync(to_free, s);
    return st;
}

// Structured body of a 2x2 matrix (m: re/im interleaved, row-major) and the
// integer-pipe multipliers its complex128 body uses.
int body_of_2x2_host(const double *mm, KConst *kc) {
    const Cm a{mm[0], mm[1]}, b{mm[2], mm[3]}, c{mm[4], mm[5]}, d{mm[6], mm[7]};
    for (int i = 0; i < 4; i++) kc[i] = make_kconst(0.0);
    const bool diag = eq(b, 0, 0) && eq(c, 0, 0);
    const bool anti = eq(a, 0, 0) && eq(d, 0, 0);
    const bool real = a.im == 0 && b.im == 0 && c.im == 0 && d.im == 0;
    const bool rxlike = a.im == 0 && d.im == 0 && a.re == d.re && b.re == 0 && c.re == 0;
    if (diag) {
        kc[0] = make_kconst(-a.im); kc[1] = make_kconst(a.im);
        kc[2] = make_kconst(-d.im); kc[3] = make_kconst(d.im);
        return B_DIAG;
    }
    if (anti && eq(b, 1, 0) && eq(c, 1, 0)) return B_PERM;
    if (anti) {
        kc[0] = make_kconst(-b.im); kc[1] = make_kconst(b.im);
        kc[2] = make_kconst(-c.im); kc[3] = make_kconst(c.im);
        return B_ANTIDIAG;
    }
    if (real) {
        kc[0] = make_kconst(b.re); kc[1] = make_kconst(c.re);
        return B_REAL;
    }
    if (rxlike) {
        kc[0] = make_kconst(-b.im); kc[1] = make_kconst(b.im);
        kc[2] = make_kconst(-c.im); kc[3] = make_kconst(c.im);
        return B_RXLIKE;
    }
    kc[0] = make_kconst(a.im); kc[1] = make_kconst(b.im);
    kc[2] = make_kconst(c.im); kc[3] = make_kconst(d.im);
    return B_DENSE;
}

template <class T, class I, bool EMU, int NT, int STAGES, int MINB, bool DFM = false>
static lgpu_status_t launch_fused_nt(cplx_t<T> *sv, const FusedParams<T, I> &p, size_t smem, cudaStream_t s) {
    static std::atomic<size_t> attr[64];
    LGPU_TRY(ensure_smem(reinterpret_cast<const void *>(fused_kernel<T, I, EMU, NT, STAGES, MINB, DFM>), smem, attr));
    const int per_sm = std::max(1, std::min(int((220 * 1024) / smem), 2048 / NT));
    const unsigned grid = unsigned(std::min<uint64_t>(uint64_t(p.ntiles), uint64_t(sm_count()) * per_sm));
    fused_kernel<T, I, EMU, NT, STAGES, MINB, DFM><<<grid, NT, smem, s>>>(sv, p);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "fused kernel launch");
    return LGPU_OK;
}

// complex64 (instruction-bound): two tile buffers per CTA, the next tile
// loading while the current one computes.  complex128 (FP64-bound): one
// buffer, three CTAs per SM interleave instead.  512 threads when only one
// CTA fits on an SM.  (Three stages with two CTAs per SM measured slower:
// the warps of a third CTA hide the tile's barrier and shared-memory
// latency better than deeper prefetch does.)
template <class T, class I, bool EMU>
static lgpu_status_t launch_fused(cplx_t<T> *sv, const FusedParams<T, I> &p, size_t tile_bytes, cudaStream_t s) {
    if constexpr (sizeof(T) == 4) {
        const size_t smem = 2 * tile_bytes;
        return smem > 64 * 1024 ? launch_fused_nt<T, I, EMU, 512, 2, 1>(sv, p, smem, s)
                                : launch_fused_nt<T, I, EMU, 256, 2, 3>(sv, p, smem, s);
    } else {
        return tile_bytes > 64 * 1024 ? launch_fused_nt<T, I, EMU, 512, 1, 1>(sv, p, tile_bytes, s)
                                      : launch_fused_nt<T, I, EMU, 256, 1, 3>(sv, p, tile_bytes, s);
    }
}

// complex128 blocks with float-float 1-target bodies.
template <class I>
static lgpu_status_t launch_fused_df(double2 *sv, const FusedParams<double, I> &p, size_t tile_bytes,
                                     cudaStream_t s) {
    const size_t smem = tile_bytes + kDiagTableBytes;  // the phase-table area after the tile
    return tile_bytes > 64 * 1024 ? launch_fused_nt<double, I, false, 512, 1, 1, true>(sv, p, smem, s)
                                  : launch_fused_nt<double, I, false, 256, 1, 3, true>(sv, p, smem, s);
}

template <class T, class I>
static lgpu_status_t fused_t(cplx_t<T> *sv, uint32_t n, const std::vector<int> &tile_bits,
                             uint32_t ngates, const lgpu_fused_gate_t *gates, uint32_t ff_flags, cudaStream_t s) {
    static_assert(sizeof(FusedParams<T, I>) <= 32000, "fused kernel parameters exceed the 32 KB limit");
    const int k = int(tile_bits.size());
    // Tile position of each state bit
    std::vector<int> pos(n, -1);
    for (int q = 0; q < k; q++) pos[size_t(tile_bits[size_t(q)])] = q;
    int m = 0;
    while (m < k && tile_bits[size_t(m)] == m) m++;
    if (k - m > 8) return fail(LGPU_ERR_INVALID_ARG, "fused tile: at most 8 tile bits above the contiguous low run");
    auto *p = new FusedParams<T, I>();
    p->holes = make_holes(tile_bits);
    p->ntiles = I(uint64_t(1) << (n - k));
    p->k = k;
    p->m = m;
    for (int h = 0; h < (1 << (k - m)); h++) {
        uint64_t o = 0;
        for (int q = m; q < k; q++)
            if ((h >> (q - m)) & 1) o |= uint64_t(1) << tile_bits[size_t(q)];
        p->hi_off[h] = I(o);
    }
    const bool emu = sizeof(T) == 8 && f64_mode() == 1;
    const bool dfm = sizeof(T) == 8 && f64_mode() == 1 && fused_df_enabled();
    std::unique_ptr<FusedParams<T, I>> guard(p);
    if (!dfm && (ff_flags & LGPU_FF_IN))  // the complex128 kernels need complex128 amplitudes
        LGPU_TRY(lgpu_state_ff(sv, n, 0, reinterpret_cast<lgpu_stream_t>(s)));
    // float-float blocks: diagonal gates folded into phase tables
    std::vector<char> internal;
    std::vector<lgpu_fused_gate_t> folded;
    if (dfm && fused_diag_fold_enabled()) {
        folded = fold_diagonal_gates(gates, ngates, pos, internal, fused_diag_fold_enabled() == 2);
        gates = folded.data();
        ngates = uint32_t(folded.size());
    }
    uint32_t done = 0;
    lgpu_status_t st = LGPU_OK;
    while (done < ngates && st == LGPU_OK) {
        int cnt = 0;
        uint32_t pool = 0;
        while (done + cnt < ngates && cnt < kFusedMaxGates) {
            const lgpu_fused_gate_t &src = gates[done + cnt];
            const uint32_t need = src.ntgt == 1 ? 8u : 32u;
            if (pool + need > uint32_t(kFusedMatPool)) break;
            FGate &dst = p->gates[cnt];
            dst = FGate{};
            dst.ntgt = uint8_t(src.ntgt);
            if (!internal.empty() && internal[done + cnt]) {  // a folded phase table (see fold_diagonal_gates)
                for (int b = 0; b < src.nctrl; b++) dst.in_mask |= 1u << pos[size_t(src.ctrl[b])];
                dst.mat_off = pool;
                for (uint32_t e = 0; e < need; e++) {
                    const DF d = df_split_host(src.m[e]);
                    std::memcpy(&p->mats[pool + e], &d, sizeof(DF));
                }
                dst.body = uint8_t(B_DENSE);
                pool += need;
                cnt++;
                continue;
            }
            if (src.ntgt != 1 && src.ntgt != 2) { st = fail(LGPU_ERR_INVALID_ARG, "fused gate: 1 or 2 targets"); break; }
            for (int j = 0; j < src.ntgt; j++) {
                if (src.tgt[j] < 0 || uint32_t(src.tgt[j]) >= n || pos[size_t(src.tgt[j])] < 0) {
                    st = fail(LGPU_ERR_INVALID_ARG, "fused gate target outside the tile");
                    break;
                }
            }
            if (st != LGPU_OK) break;
            dst.q0 = uint8_t(pos[size_t(src.tgt[0])]);
            dst.q1 = src.ntgt == 2 ? uint8_t(pos[size_t(src.tgt[1])]) : 0;
            if (src.ntgt == 2 && dst.q0 == dst.q1) { st = fail(LGPU_ERR_INVALID_ARG, "fused gate: repeated target"); break; }
            if (src.nctrl < 0 || src.nctrl > 4) { st = fail(LGPU_ERR_INVALID_ARG, "fused gate: at most 4 controls"); break; }
            for (int j = 0; j < src.nctrl; j++) {
                const int b = src.ctrl[j];
                if (b < 0 || uint32_t(b) >= n) { st = fail(LGPU_ERR_INVALID_ARG, "fused gate control out of range"); break; }
                for (int q = 0; q < src.ntgt; q++)
                    if (src.tgt[q] == b) { st = fail(LGPU_ERR_INVALID_ARG, "fused gate: control equals target"); break; }
                if (st != LGPU_OK) break;
                const int v = src.ctrl_val[j] ? 1 : 0;
                if (pos[size_t(b)] >= 0) {
                    if (dst.in_mask & (1u << pos[size_t(b)])) { st = fail(LGPU_ERR_INVALID_ARG, "fused gate: repeated control"); break; }
                    dst.in_mask |= 1u << pos[size_t(b)];
                    if (v) dst.in_val |= 1u << pos[size_t(b)];
                } else {
                    dst.out_mask |= uint64_t(1) << b;
                    if (v) dst.out_val |= uint64_t(1) << b;
                }
            }
            if (st != LGPU_OK) break;
            dst.mat_off = pool;
            if (dfm) {  // (hi, lo) float pairs in the double slots
                for (uint32_t e = 0; e < need; e++) {
                    const DF d = df_split_host(src.m[e]);
                    std::memcpy(&p->mats[pool + e], &d, sizeof(DF));
                }
            } else {
                for (uint32_t e = 0; e < need; e++) p->mats[pool + e] = T(src.m[e]);
            }
            dst.body = src.ntgt == 1 ? uint8_t(body_of_2x2_host(src.m, p->kc[cnt])) : uint8_t(B_DENSE);
            dst.pad = (dfm && src.ntgt == 1 && df_sign_diag_host(src.m)) ? 1 : 0;  // float-float sign flips
            pool += need;
            cnt++;
        }
        if (st != LGPU_OK) break;
        p->ngates = cnt;
        p->ngroups = group_fused_gates(p->gates, p->kc, cnt, sizeof(T) == 4 ? k : 0, fused_reg_bits<T>(), p->groups);
        // float-float path: the first launch reads the state as it arrives, the
        // last leaves it as asked, launches in between keep float-float
        p->in_ff = dfm && (done > 0 || (ff_flags & LGPU_FF_IN)) ? 1 : 0;
        p->out_ff = dfm && (done + uint32_t(cnt) < ngates || (ff_flags & LGPU_FF_OUT)) ? 1 : 0;
        const size_t smem = (size_t(1) << k) * sizeof(cplx_t<T>);
        if constexpr (sizeof(T) == 8)
            st = dfm ? launch_fused_df<I>(sv, *p, smem, s)
                     : emu ? launch_fused<T, I, true>(sv, *p, smem, s) : launch_fused<T, I, false>(sv, *p, smem, s);
        else
            st = launch_fused<T, I, false>(sv, *p, smem, s);
        done += uint32_t(cnt);
    }
    if (st == LGPU_OK && !dfm && (ff_flags & LGPU_FF_OUT))
        st = lgpu_state_ff(sv, n, 1, reinterpret_cast<lgpu_stream_t>(s));
    return st;
}

}  // namespace lgpu

namespace lgpu {

// Stream -> error slot: the legacy and per-thread default streams (handles
// 0, 1, 2) use slot 0; other streams get slots 1 .. kErrSlots - 1 in order of
// first use, and share them round-robin beyond that.
static std::mutex g_err_mu;
static std::unordered_map<uintptr_t, int> g_err_slot;
static int g_err_next = 0;
static std::atomic<unsigned *> g_err_base[64];
static std::atomic<unsigned> g_err_epoch[64];

lgpu_status_t stream_error_ptr(cudaStream_t s, unsigned **out) {
    int dev = 0;
    LGPU_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return fail(LGPU_ERR_UNSUPPORTED, "device ordinal beyond 63");
    const uintptr_t h = reinterpret_cast<uintptr_t>(s);
    std::lock_guard<std::mutex> lock(g_err_mu);
    int slot = 0;
    if (h > 2) {
        auto it = g_err_slot.find(h);
        if (it == g_err_slot.end()) {
            slot = 1 + (g_err_next++ % (kErrSlots - 1));
            g_err_slot.emplace(h, slot);
        } else {
            slot = it->second;
        }
    }
    unsigned *base = g_err_base[dev].load(std::memory_order_acquire);
    if (!base || g_err_epoch[dev].load(std::memory_order_acquire) != reset_epoch()) {
        void *p = nullptr;
        LGPU_CUDA_TRY(cudaGetSymbolAddress(&p, g_lgpu_stream_error));
        base = static_cast<unsigned *>(p);
        g_err_base[dev].store(base, std::memory_order_release);
        g_err_epoch[dev].store(reset_epoch(), std::memory_order_release);
    }
    *out = base + slot;
    return LGPU_OK;
}

}  // namespace lgpu

using namespace lgpu;

extern "C" {

lgpu_status_t lgpu_selftest_bounded_wait(uint32_t spin_limit, lgpu_stream_t stream) {
    if (spin_limit == 0 || spin_limit > kWaitLimit) return fail(LGPU_ERR_INVALID_ARG, "spin limit out of range");
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    unsigned *err = nullptr;
    LGPU_TRY(stream_error_ptr(s, &err));
    wait_selftest_kernel<<<1, 64, 0, s>>>(spin_limit, err);
    LGPU_CHECK_LAUNCH();
    LGPU_CUDA_TRY(cudaStreamSynchronize(s));
    return LGPU_OK;
}

lgpu_status_t lgpu_device_error(int *code, int reset) {
    if (!code) return fail(LGPU_ERR_INVALID_ARG, "code is null");
    unsigned v = 0, vb = 0;
    LGPU_CUDA_TRY(cudaMemcpyFromSymbol(&v, g_lgpu_device_error, sizeof(v)));
    LGPU_TRY(batch_error_fetch(&vb, reset != 0));
    *code = int(v | vb);
    if (reset && v) {
        unsigned z = 0;
        LGPU_CUDA_TRY(cudaMemcpyToSymbol(g_lgpu_device_error, &z, sizeof(z)));
    }
    return LGPU_OK;
}

lgpu_status_t lgpu_stream_error(lgpu_stream_t stream, int *code, int reset) {
    if (!code) return fail(LGPU_ERR_INVALID_ARG, "code is null");
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    unsigned *err = nullptr;
    LGPU_TRY(stream_error_ptr(s, &err));
    unsigned v = 0;
    LGPU_CUDA_TRY(cudaMemcpyAsync(&v, err, sizeof(v), cudaMemcpyDeviceToHost, s));
    LGPU_CUDA_TRY(cudaStreamSynchronize(s));
    *code = int(v);
    if (reset && v) {
        LGPU_CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(unsigned), s));
        LGPU_CUDA_TRY(cudaStreamSynchronize(s));
    }
    return LGPU_OK;
}

lgpu_status_t lgpu_apply_matrix(void *sv, uint32_t n, lgpu_dtype_t dt, const double *matrix, uint32_t t,
                                const int32_t *tgts, uint32_t c, const int32_t *ctrls,
                                const int32_t *ctrl_vals, int adjoint, lgpu_stream_t stream) {
    LGPU_TRY(check_state(sv, n, dt));
    if (!matrix) return fail(LGPU_ERR_INVALID_ARG, "matrix is null");
    GateGeometry g;
    LGPU_TRY(geometry(n, t, tgts, c, ctrls, ctrl_vals, &g));
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    return dt == LGPU_C128 ? apply_matrix_dispatch<double>(sv, nullptr, 0, n, matrix, t, g, adjoint, s)
                           : apply_matrix_dispatch<float>(sv, nullptr, 0, n, matrix, t, g, adjoint, s);
}

lgpu_status_t lgpu_apply_matrix_multi(void *const *svs, uint32_t nstates, uint32_t n, lgpu_dtype_t dt,
                                      const double *matrix, uint32_t t, const int32_t *tgts, uint32_t c,
                                      const int32_t *ctrls, const int32_t *ctrl_vals, int adjoint,
                                      lgpu_stream_t stream) {
    if (nstates == 0) return LGPU_OK;
    if (!svs) return fail(LGPU_ERR_INVALID_ARG, "state array is null");
    if (nstates > 65535) return fail(LGPU_ERR_INVALID_ARG, "too many states in one launch");
    for (uint32_t k = 0; k < nstates; k++) LGPU_TRY(check_state(svs[k], n, dt));
    if (!matrix) return fail(LGPU_ERR_INVALID_ARG, "matrix is null");
    GateGeometry g;
    LGPU_TRY(geometry(n, t, tgts, c, ctrls, ctrl_vals, &g));
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    return dt == LGPU_C128 ? apply_matrix_dispatch<double>(nullptr, svs, nstates, n, matrix, t, g, adjoint, s)
                           : apply_matrix_dispatch<float>(nullptr, svs, nstates, n, matrix, t, g, adjoint, s);
}

lgpu_status_t lgpu_apply_pauli_rotation(void *sv, uint32_t n, lgpu_dtype_t dt, double angle, uint32_t t,
                                        const int32_t *tgts, const char *paulis, uint32_t c,
                                        const int32_t *ctrls, const int32_t *ctrl_vals,
                                        lgpu_stream_t stream) {
    LGPU_TRY(check_state(sv, n, dt));
    if (!paulis) return fail(LGPU_ERR_INVALID_ARG, "paulis is null");
    if (t < 1 || t > n) return fail(LGPU_ERR_INVALID_ARG, "bad number of Pauli targets");
    GateGeometry g;
    if (c > LGPU_MAX_CONTROLS) return fail(LGPU_ERR_INVALID_ARG, "too many controls");
    LGPU_TRY(check_bits(n, t, tgts, "target", &g.tgts));
    LGPU_TRY(check_bits(n, c, ctrls, "control", &g.ctrls));
    std::vector<int> all(g.tgts);
    all.insert(all.end(), g.ctrls.begin(), g.ctrls.end());
    std::sort(all.begin(), all.end());
    if (std::adjacent_find(all.begin(), all.end()) != all.end())
        return fail(LGPU_ERR_INVALID_ARG, "target and control bits must be distinct");
    for (uint32_t k = 0; k < c; k++) {
        const int v = ctrl_vals ? ctrl_vals[k] : 1;
        g.cvals.push_back(v);
        if (v) g.cset |= uint64_t(1) << g.ctrls[k];
    }
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    return dt == LGPU_C128 ? pauli_rot_dispatch<double>(sv, nullptr, 0, n, angle, g, paulis, s)
                           : pauli_rot_dispatch<float>(sv, nullptr, 0, n, angle, g, paulis, s);
}

lgpu_status_t lgpu_apply_pauli_rotation_multi(void *const *svs, uint32_t nstates, uint32_t n, lgpu_dtype_t dt,
                                              double angle, uint32_t t, const int32_t *tgts,
                                              const char *paulis, uint32_t c, const int32_t *ctrls,
                                              const int32_t *ctrl_vals, lgpu_stream_t stream) {
    if (nstates == 0) return LGPU_OK;
    if (!svs || !paulis) return fail(LGPU_ERR_INVALID_ARG, "null argument");
    if (nstates > 65535) return fail(LGPU_ERR_INVALID_ARG, "too many states in one launch");
    for (uint32_t k = 0; k < nstates; k++) LGPU_TRY(check_state(svs[k], n, dt));
    if (t < 1 || t > n) return fail(LGPU_ERR_INVALID_ARG, "bad number of Pauli targets");
    GateGeometry g;
    if (c > LGPU_MAX_CONTROLS) return fail(LGPU_ERR_INVALID_ARG, "too many controls");
    LGPU_TRY(check_bits(n, t, tgts, "target", &g.tgts));
    LGPU_TRY(check_bits(n, c, ctrls, "control", &g.ctrls));
    std::vector<int> all(g.tgts);
    all.insert(all.end(), g.ctrls.begin(), g.ctrls.end());
    std::sort(all.begin(), all.end());
    if (std::adjacent_find(all.begin(), all.end()) != all.end())
        return fail(LGPU_ERR_INVALID_ARG, "target and control bits must be distinct");
    for (uint32_t k = 0; k < c; k++) {
        const int v = ctrl_vals ? ctrl_vals[k] : 1;
        g.cvals.push_back(v);
        if (v) g.cset |= uint64_t(1) << g.ctrls[k];
    }
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    return dt == LGPU_C128 ? pauli_rot_dispatch<double>(nullptr, svs, nstates, n, angle, g, paulis, s)
                           : pauli_rot_dispatch<float>(nullptr, svs, nstates, n, angle, g, paulis, s);
}

lgpu_status_t lgpu_apply_fused_block(void *sv, uint32_t n, lgpu_dtype_t dt, uint32_t k,
                                     const int32_t *tile_bits, uint32_t ngates,
                                     const lgpu_fused_gate_t *gates, lgpu_stream_t stream) {
    return lgpu_apply_fused_block_ff(sv, n, dt, k, tile_bits, ngates, gates, 0, stream);
}

lgpu_status_t lgpu_apply_fused_block_ff(void *sv, uint32_t n, lgpu_dtype_t dt, uint32_t k,
                                        const int32_t *tile_bits, uint32_t ngates,
                                        const lgpu_fused_gate_t *gates, uint32_t ff_flags, lgpu_stream_t stream) {
    LGPU_TRY(check_state(sv, n, dt));
    if (ff_flags & ~uint32_t(LGPU_FF_IN | LGPU_FF_OUT)) return fail(LGPU_ERR_INVALID_ARG, "fused block: unknown flags");
    if (ff_flags && dt != LGPU_C128)
        return fail(LGPU_ERR_INVALID_ARG, "fused block: float-float states are complex128 only");
    if (ngates == 0) {  // nothing to apply; the state still takes the requested form
        const bool in = (ff_flags & LGPU_FF_IN) != 0, out = (ff_flags & LGPU_FF_OUT) != 0;
        if (in != out) return lgpu_state_ff(sv, n, out ? 1 : 0, stream);
        return LGPU_OK;
    }
    if (!gates) return fail(LGPU_ERR_INVALID_ARG, "gates is null");
    const uint32_t kmax = dt == LGPU_C128 ? 12u : 13u;
    if (k < 1 || k > kmax || k > n)
        return fail(LGPU_ERR_INVALID_ARG, "fused tile size out of range");
    std::vector<int> tb;
    LGPU_TRY(check_bits(n, k, tile_bits, "tile", &tb));
    std::sort(tb.begin(), tb.end());
    if (std::adjacent_find(tb.begin(), tb.end()) != tb.end())
        return fail(LGPU_ERR_INVALID_ARG, "tile bits must be distinct");
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    if (dt == LGPU_C128)
        return n <= 32 ? fused_t<double, uint32_t>(static_cast<double2 *>(sv), n, tb, ngates, gates, ff_flags, s)
                       : fused_t<double, uint64_t>(static_cast<double2 *>(sv), n, tb, ngates, gates, ff_flags, s);
    return n <= 32 ? fused_t<float, uint32_t>(static_cast<float2 *>(sv), n, tb, ngates, gates, 0, s)
                   : fused_t<float, uint64_t>(static_cast<float2 *>(sv), n, tb, ngates, gates, 0, s);
}

}  // extern "C"
