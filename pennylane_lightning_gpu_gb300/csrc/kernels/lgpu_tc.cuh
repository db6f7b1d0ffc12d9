// Dense 6-qubit gates on the tensor cores (tcgen05, sm_103a), complex64.
//
// A dense 64 x 64 complex matrix U on the six lowest state bits maps every
// run of 64 consecutive amplitudes (a "column" of the state) to U times that
// run.  In real arithmetic a column is 128 floats (re, im interleaved) and U
// is the 128 x 128 real matrix R with 2x2 blocks [[ur, -ui], [ui, ur]], so a
// tile of 64 consecutive columns (4096 amplitudes, 32 KB) is one GEMM
//     D (128 x 64) = R (128 x 128) . X (128 x 64)
// with M = 128 output reals, N = 64 columns, K = 128 input reals.
//
// Precision: three TF32 products with FP32 accumulation in tensor memory,
// D = Rhi.Xhi + Rhi.Xlo + Rlo.Xhi, where hi = TF32 rounding of the float and
// lo = TF32 rounding of the remainder (Rlo.Xlo, about 2^-22 relative, is
// dropped).  The error per output is a few FP32 ulps of the column's size.
//
// One persistent CTA per SM (256 threads, 224 KB of shared memory), tiles of
// 64 columns (4096 amplitudes, 32 KB):
//   R hi / lo      : 2 x 64 KB, built once from U (A operands, K-major)
//   X hi / lo      : 2 x 32 KB, rebuilt per tile (B operands, K-major, N = 64)
//   staging        : 32 KB, the next tile lands here by one cp.async.bulk
//   D              : two slots of 64 TMEM columns
// While the tensor core multiplies tile j into D slot j & 1, the CTA reads out
// and stores tile j - 1 from the other slot; the load of tile j + 1 is issued
// with the MMAs of tile j.  The operand descriptors are built once; a K step
// adds 256 bytes (16 in the address field) to them.
// Operands use the no-swizzle canonical layout: core matrices of 8 rows x 16
// bytes (128 contiguous bytes), 32 of them along K per group of 8 rows
// (LBO = 128 B between K-neighbours, SBO = 4096 B between row groups).
// Warp w reads TMEM lanes 32 (w % 4) .. + 31 (output reals) of 32 of the 64
// columns and stores them: for each column the warp writes 128 contiguous
// bytes.
//
// Every wait (a tile's bulk copy, an MMA commit) is bounded; a CTA that gives
// up records it in its stream's error word and the device-wide flag, waits
// (bounded again) for the copies and MMAs it issued, frees its tensor memory
// and leaves.
#pragma once

namespace lgpu {

constexpr int kTcThreads = 256;
constexpr int kTcCols = 64;   // state columns per tile (N)
constexpr int kTcK = 128;     // real inputs per column (K)
constexpr int kTcM = 128;     // real outputs per column (M)
constexpr uint32_t kTcTmemCols = 128;  // two D slots of kTcCols columns
constexpr uint32_t kTcGroupBytes = (kTcK / 4) * 128;  // one group of 8 rows: 32 core matrices
constexpr uint32_t kTcRBytes = (kTcM / 8) * kTcGroupBytes;     // 64 KB
constexpr uint32_t kTcXBytes = (kTcCols / 8) * kTcGroupBytes;  // 32 KB
constexpr uint32_t kTcTileBytes = kTcCols * 64 * 8;            // 32 KB of complex64 amplitudes
constexpr uint32_t kTcTileAmps = kTcCols * 64;
constexpr size_t kTcSmemBytes = 2 * size_t(kTcRBytes) + 2 * size_t(kTcXBytes) + size_t(kTcTileBytes);  // 224 KB

// Byte offset of element (row, k) in a K-major no-swizzle operand.
__host__ __device__ __forceinline__ uint32_t tc_off(uint32_t row, uint32_t k) {
    return (row >> 3) * kTcGroupBytes + (k >> 2) * 128u + (row & 7u) * 16u + (k & 3u) * 4u;
}

// Shared-memory matrix descriptor (tcgen05): start address, leading (K)
// byte offset, stride (row-group) byte offset, descriptor version 1, no
// swizzle, base offset 0.
__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr) {
    return uint64_t((saddr >> 4) & 0x3FFFu) | (uint64_t((128u >> 4) & 0x3FFFu) << 16) |
           (uint64_t((kTcGroupBytes >> 4) & 0x3FFFu) << 32) | (uint64_t(1) << 46);
}

// Instruction descriptor, kind::tf32: D = F32, A = B = TF32, both K-major,
// N = 64, M = 128.
constexpr uint32_t kTcIdesc = (1u << 4) | (2u << 7) | (2u << 10) | (uint32_t(kTcCols >> 3) << 17) |
                              (uint32_t(kTcM >> 4) << 24);

__device__ __forceinline__ float tc_tf32(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}

__device__ __forceinline__ void tc_mma(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(kTcIdesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void tc_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// 16 consecutive TMEM columns of this warp's 32 lanes.
__device__ __forceinline__ void tc_ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void tc_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// Bounded wait on an mbarrier phase; true when it completed.
__device__ __forceinline__ bool tc_wait(uint64_t *bar, uint32_t parity) {
    for (uint32_t spins = 0; spins <= kWaitLimit; spins++)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

struct TcDense6Params {
    unsigned *err;      // the launch stream's error word
    const float2 *u;    // 64 x 64 row-major, rows / columns in state-bit order (bit 0 = LSB)
    uint64_t ntiles;    // 2^n / 4096
};

__global__ void __launch_bounds__(kTcThreads, 1) dense6_tc_kernel(float2 *__restrict__ sv, const TcDense6Params p) {
    extern __shared__ __align__(1024) unsigned char tc_smem[];
    __shared__ __align__(8) uint64_t bar_load, bar_mma[2];
    __shared__ uint32_t tmem_slot;
    unsigned char *r_hi = tc_smem;
    unsigned char *r_lo = tc_smem + kTcRBytes;
    unsigned char *x_hi = tc_smem + 2 * kTcRBytes;
    unsigned char *x_lo = x_hi + kTcXBytes;
    float4 *stage = reinterpret_cast<float4 *>(x_lo + kTcXBytes);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint64_t G = gridDim.x;
    const uint64_t J = p.ntiles > blockIdx.x ? (p.ntiles - blockIdx.x + G - 1) / G : 0;  // tiles of this CTA

    if (tid == 0) {
        mbar_init(&bar_load, 1);
        mbar_init(&bar_mma[0], 1);
        mbar_init(&bar_mma[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                     "r"(kTcTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
        tc_fence_before();
    }
    // R (hi, lo) from U: entry (m, k) with m = 2r + a, k = 2c + b
    for (int e = tid; e < kTcM * kTcK; e += kTcThreads) {
        const int m = e / kTcK, k = e % kTcK;
        const float2 u = p.u[(m >> 1) * 64 + (k >> 1)];
        const int a = m & 1, b = k & 1;
        const float v = a == b ? u.x : (a ? u.y : -u.y);
        const float hi = tc_tf32(v);
        *reinterpret_cast<float *>(r_hi + tc_off(uint32_t(m), uint32_t(k))) = hi;
        *reinterpret_cast<float *>(r_lo + tc_off(uint32_t(m), uint32_t(k))) = tc_tf32(v - hi);
    }
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_slot;
    const uint64_t d_rh = tc_desc(smem_u32(r_hi)), d_rl = tc_desc(smem_u32(r_lo));
    const uint64_t d_xh = tc_desc(smem_u32(x_hi)), d_xl = tc_desc(smem_u32(x_lo));

    auto tile_ptr = [&](uint64_t j) { return sv + (blockIdx.x + j * G) * uint64_t(kTcTileAmps); };
    auto issue_load = [&](uint64_t j) {
        mbar_expect_tx(&bar_load, kTcTileBytes);
        bulk_load(stage, tile_ptr(j), kTcTileBytes, &bar_load);
    };
    // Read out D of tile j (slot j & 1) and store it: warp w takes lanes
    // 32 (w % 4) .. + 31 and columns 32 (w / 4) .. + 31.
    auto store_tile = [&](uint64_t j) {
        const int q = int(j & 1);
        float *dst = reinterpret_cast<float *>(tile_ptr(j));
        const uint32_t row = uint32_t((warp & 3) * 32 + lane);
        const uint32_t taddr = tmem + (uint32_t((warp & 3) * 32) << 16) + uint32_t(q * kTcCols);
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const int c0 = (warp >> 2) * 32 + h * 16;
            float v[16];
            tc_ld16(taddr + uint32_t(c0), v);
            tc_wait_ld();
#pragma unroll
            for (int i = 0; i < 16; i++) __stcs(dst + size_t(c0 + i) * kTcK + row, v[i]);
        }
    };
    // issue / wait bookkeeping (thread 0 issues; everyone waits): the load of
    // tile j completes phase j & 1 of bar_load; the MMA batch of tile j
    // completes phase (j >> 1) & 1 of bar_mma[j & 1]
    uint64_t loads_issued = 0, loads_done = 0, mmas_issued = 0, mmas_done = 0;
    if (tid == 0 && J > 0) issue_load(0);
    loads_issued = J > 0 ? 1 : 0;

    bool failed = false;
    for (uint64_t j = 0; j < J; j++) {
        if (j >= 1) {  // X is reused: the MMAs of tile j - 1 must be done
            const uint64_t jp = j - 1;
            if (__syncthreads_or(!tc_wait(&bar_mma[jp & 1], uint32_t((jp >> 1) & 1))))  {
                failed = true;
                break;
            }
            mmas_done = j;
        }
        if (__syncthreads_or(!tc_wait(&bar_load, uint32_t(j & 1)))) {
            failed = true;
            break;
        }
        loads_done = j + 1;
        // staging -> X hi / lo.  Lane L takes column 8 (w % 8) + (L & 7) and
        // the 16-byte chunks (4 t + (L >> 3) + (L & 7)) mod 32, t = 0..7:
        // conflict-free reads (8 distinct chunk slots per phase) and writes
        // (8 rows of one core matrix).
        {
            const int col = warp * 8 + (lane & 7);
#pragma unroll
            for (int t = 0; t < 8; t++) {
                const int chunk = (4 * t + (lane >> 3) + (lane & 7)) & 31;  // 4 reals
                const float4 x = stage[col * 32 + chunk];
                float4 h, l;
                h.x = tc_tf32(x.x);
                l.x = tc_tf32(x.x - h.x);
                h.y = tc_tf32(x.y);
                l.y = tc_tf32(x.y - h.y);
                h.z = tc_tf32(x.z);
                l.z = tc_tf32(x.z - h.z);
                h.w = tc_tf32(x.w);
                l.w = tc_tf32(x.w - h.w);
                const uint32_t o = tc_off(uint32_t(col), uint32_t(chunk * 4));
                *reinterpret_cast<float4 *>(x_hi + o) = h;
                *reinterpret_cast<float4 *>(x_lo + o) = l;
            }
        }
        fence_async_shared();  // the operands are read by the tensor core (async proxy)
        __syncthreads();
        if (tid == 0) {
            if (j + 1 < J) issue_load(j + 1);  // the staging buffer is free: every thread has read it
            tc_fence_after();
            const uint32_t d = tmem + uint32_t(int(j & 1) * kTcCols);
#pragma unroll 1
            for (uint32_t ks = 0; ks < kTcK / 8; ks++) {  // 8 reals = 32 bytes = two core matrices along K
                const uint64_t o = uint64_t(ks) * 16u;    // 256 bytes in the address field (16-byte units)
                tc_mma(d, d_rh + o, d_xh + o, ks > 0);
                tc_mma(d, d_rh + o, d_xl + o, 1u);
                tc_mma(d, d_rl + o, d_xh + o, 1u);
            }
            tc_commit(&bar_mma[j & 1]);
        }
        loads_issued = j + 1 < J ? j + 2 : J;
        mmas_issued = j + 1;
        if (j >= 1) {  // tile j - 1 (its MMAs are done) while the tensor core works on tile j
            tc_fence_after();
            store_tile(j - 1);
        }
        tc_fence_before();
        __syncthreads();  // D slot (j - 1) & 1 is free for tile j + 1
    }
    if (!failed && J > 0) {
        const uint64_t jl = J - 1;
        if (__syncthreads_or(!tc_wait(&bar_mma[jl & 1], uint32_t((jl >> 1) & 1)))) {
            failed = true;
        } else {
            mmas_done = J;
            tc_fence_after();
            store_tile(jl);
        }
    }
    if (failed && tid == 0) {
        report_timeout(p.err);
        for (uint64_t j = loads_done; j < loads_issued; j++) tc_wait(&bar_load, uint32_t(j & 1));
        for (uint64_t j = mmas_done; j < mmas_issued; j++) tc_wait(&bar_mma[j & 1], uint32_t((j >> 1) & 1));
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTcTmemCols)
                     : "memory");
    }
}

}  // namespace lgpu
