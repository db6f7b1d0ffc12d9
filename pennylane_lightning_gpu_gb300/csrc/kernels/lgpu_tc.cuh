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
// One persistent CTA per SM (9 warps, 192 KB of shared memory, all 512 TMEM
// columns), tiles of 64 columns (4096 amplitudes, 32 KB):
//   R hi / lo      : TMEM columns 0..127 / 128..255, written once from U
//                    (the A operand comes from tensor memory: row m in lane m)
//   D              : TMEM columns 256..383, two slots of 64
//   X hi / lo      : two slots of 2 x 32 KB of shared memory (B operands,
//                    K-major, N = 64)
//   staging        : two slots of 32 KB, tiles land here by cp.async.bulk
// Warp 0 is the producer: one thread issues the tile loads and the MMAs.
// Warps 1..8 are the consumers: they split tile j into X slot j & 1, then read
// out and store tile j - 1, while the tensor core multiplies tile j.  The two
// roles meet only at mbarriers (tile landed, X slot filled, MMAs done, D slot
// read out), so the MMA issue never waits behind the stores.  The B
// descriptors are built once per slot; a K step adds 256 bytes (16 in the
// address field) to them and 8 columns to the A address.
// The B operand uses the no-swizzle canonical layout: core matrices of 8 rows
// x 16 bytes (128 contiguous bytes), 32 of them along K per group of 8 rows
// (LBO = 128 B between K-neighbours, SBO = 4096 B between row groups).
// Consumer warp w reads TMEM lanes 32 (w % 4) .. + 31 (output reals) of 32 of
// the 64 columns of a D slot and stores them: for each column the warp writes
// 128 contiguous bytes.
//
// Every wait is bounded; a thread that gives up marks the CTA failed, which
// the other role sees at its next wait.  The CTA then records the time-out in
// its stream's error word and the device-wide flag, waits (bounded again) for
// the copies and MMAs it issued, frees its tensor memory and leaves.
#pragma once

namespace lgpu {

constexpr int kTcThreads = 288;  // warp 0: producer; warps 1..8: consumers
constexpr int kTcCols = 64;   // state columns per tile (N)
constexpr int kTcK = 128;     // real inputs per column (K)
constexpr int kTcM = 128;     // real outputs per column (M)
constexpr uint32_t kTcTmemCols = 512;                   // R hi, R lo, two D slots
constexpr uint32_t kTcTmemRlo = kTcK, kTcTmemD = 2 * kTcK;  // column offsets
constexpr uint32_t kTcGroupBytes = (kTcK / 4) * 128;  // one group of 8 rows: 32 core matrices
constexpr uint32_t kTcXBytes = (kTcCols / 8) * kTcGroupBytes;  // 32 KB
constexpr uint32_t kTcTileBytes = kTcCols * 64 * 8;            // 32 KB of complex64 amplitudes
constexpr uint32_t kTcTileAmps = kTcCols * 64;
constexpr size_t kTcSmemBytes = 4 * size_t(kTcXBytes) + 2 * size_t(kTcTileBytes);  // 192 KB

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

// TF32 rounding (nearest, ties away from zero) of a finite float with two
// integer operations: add half a TF32 ulp to the magnitude bits, clear the 13
// low mantissa bits (a carry into the exponent is the correct rounding up).
// The same bits as cvt.rna.tf32.f32, which runs on a slower conversion pipe.
__device__ __forceinline__ float tc_tf32(float x) {
    return __uint_as_float((__float_as_uint(x) + 0x1000u) & 0xFFFFE000u);
}

// D (TMEM) (+)= A (TMEM, row m in lane m, K along columns) . B (shared memory)
__device__ __forceinline__ void tc_mma_ts(uint32_t d_tmem, uint32_t a_tmem, uint64_t bdesc, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], [%1], %2, %3, p;\n\t}" ::"r"(d_tmem),
        "r"(a_tmem), "l"(bdesc), "r"(kTcIdesc), "r"(accumulate)
        : "memory");
}

// 16 consecutive TMEM columns of this warp's 32 lanes from registers.
__device__ __forceinline__ void tc_st16(uint32_t taddr, const float (&v)[16]) {
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15, %16};" ::"r"(taddr),
        "r"(__float_as_uint(v[0])), "r"(__float_as_uint(v[1])), "r"(__float_as_uint(v[2])), "r"(__float_as_uint(v[3])),
        "r"(__float_as_uint(v[4])), "r"(__float_as_uint(v[5])), "r"(__float_as_uint(v[6])), "r"(__float_as_uint(v[7])),
        "r"(__float_as_uint(v[8])), "r"(__float_as_uint(v[9])), "r"(__float_as_uint(v[10])),
        "r"(__float_as_uint(v[11])), "r"(__float_as_uint(v[12])), "r"(__float_as_uint(v[13])),
        "r"(__float_as_uint(v[14])), "r"(__float_as_uint(v[15]))
        : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void tc_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }

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
    // per slot q: tile landed (tx), X filled (8 consumer warps), MMAs done
    // (commit), D read out (8 consumer warps)
    __shared__ __align__(8) uint64_t bar_load[2], bar_x[2], bar_mma[2], bar_dfree[2];
    __shared__ uint32_t tmem_slot;
    __shared__ volatile int s_failed;
    unsigned char *xbuf = tc_smem;  // slot q: hi at 2 q X, lo at (2 q + 1) X
    float4 *stage = reinterpret_cast<float4 *>(tc_smem + 4 * kTcXBytes);  // slot q at q * (tile / 16 B)
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint64_t G = gridDim.x;
    const uint64_t J = p.ntiles > blockIdx.x ? (p.ntiles - blockIdx.x + G - 1) / G : 0;  // tiles of this CTA

    if (tid == 0) {
        for (int q = 0; q < 2; q++) {
            mbar_init(&bar_load[q], 1);
            mbar_init(&bar_x[q], 8);
            mbar_init(&bar_mma[q], 1);
            mbar_init(&bar_dfree[q], 8);
        }
        s_failed = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                     "r"(kTcTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
        tc_fence_before();
    }
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_slot;
    const uint32_t lane_base = uint32_t((warp & 3) * 32) << 16;  // this warp's TMEM lane quarter
    const int half = warp >= 1 ? (warp - 1) >> 2 : 0;            // consumer column half

    auto tile_ptr = [&](uint64_t j) { return sv + (blockIdx.x + j * G) * uint64_t(kTcTileAmps); };
    auto issue_load = [&](uint64_t j) {
        const int q = int(j & 1);
        mbar_expect_tx(&bar_load[q], kTcTileBytes);
        bulk_load(stage + size_t(q) * (kTcTileBytes / 16), tile_ptr(j), kTcTileBytes, &bar_load[q]);
    };
    // a bounded wait that gives up early once the other role has failed
    auto wait = [&](uint64_t *bar, uint64_t use) {
        const uint32_t parity = uint32_t(use & 1);
        for (uint32_t spins = 0; spins <= kWaitLimit; spins++) {
            if (mbar_try_wait(bar, parity)) return true;
            if ((spins & 1023u) == 1023u && s_failed) return false;
        }
        s_failed = 1;
        return false;
    };
    // producer bookkeeping (thread 0): loads and MMA batches issued and known complete
    uint64_t loads_issued = 0, mmas_issued = 0;

    if (tid == 0)
        for (uint64_t j = 0; j < 2 && j < J; j++) issue_load(j);
    loads_issued = J < 2 ? J : 2;

    // R (hi, lo) into TMEM by the consumers: warp w writes row m = 32 (w % 4) +
    // lane, columns 64 half .. + 63 of each; entry (m, k), m = 2r + a, k = 2c + b.
    if (warp >= 1) {
        const int m = (warp & 3) * 32 + lane, a = m & 1;
#pragma unroll 1
        for (int c0 = half * 64; c0 < half * 64 + 64; c0 += 16) {
            float hi[16], lo[16];
#pragma unroll
            for (int i = 0; i < 16; i++) {
                const int k = c0 + i, b = k & 1;
                const float2 u = p.u[(m >> 1) * 64 + (k >> 1)];
                const float v = a == b ? u.x : (a ? u.y : -u.y);
                hi[i] = tc_tf32(v);
                lo[i] = tc_tf32(v - hi[i]);
            }
            tc_st16(tmem + lane_base + uint32_t(c0), hi);
            tc_st16(tmem + lane_base + kTcTmemRlo + uint32_t(c0), lo);
        }
        tc_wait_st();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();

    if (warp == 0) {
        // ---- producer: loads two tiles ahead, MMAs of tile j once X slot j & 1
        // is filled and D slot j & 1 has been read out (tile j - 2)
        if (lane == 0) {
            for (uint64_t j = 0; j < J; j++) {
                const int q = int(j & 1);
                if (!wait(&bar_x[q], j >> 1)) break;
                if (j + 2 < J) {  // staging slot q is free: tile j has been split
                    issue_load(j + 2);
                    loads_issued = j + 3;
                }
                if (j >= 2 && !wait(&bar_dfree[q], (j - 2) >> 1)) break;
                tc_fence_after();
                const uint64_t bh = tc_desc(smem_u32(xbuf + size_t(2 * q) * kTcXBytes));
                const uint64_t bl = tc_desc(smem_u32(xbuf + size_t(2 * q + 1) * kTcXBytes));
                const uint32_t d = tmem + kTcTmemD + uint32_t(q * kTcCols);
#pragma unroll 1
                for (uint32_t ks = 0; ks < kTcK / 8; ks++) {  // 8 reals: 8 TMEM columns of A, 32 bytes of B
                    const uint64_t o = uint64_t(ks) * 16u;
                    const uint32_t ac = ks * 8u;
                    tc_mma_ts(d, tmem + ac, bh + o, ks > 0);
                    tc_mma_ts(d, tmem + ac, bl + o, 1u);
                    tc_mma_ts(d, tmem + kTcTmemRlo + ac, bh + o, 1u);
                }
                tc_commit(&bar_mma[q]);
                mmas_issued = j + 1;
            }
        }
    } else {
        // ---- consumers: split tile j, then read out and store tile j - 1
        const int cw = warp - 1;
        const uint32_t row = uint32_t((warp & 3) * 32 + lane);
        for (uint64_t j = 0; j <= J; j++) {
            if (j < J) {
                const int q = int(j & 1);
                if (!wait(&bar_load[q], j >> 1)) break;
                if (j >= 2 && !wait(&bar_mma[q], (j - 2) >> 1)) break;  // X slot q: the MMAs of tile j - 2 are done
                // staging slot q -> X slot q.  Lane L takes column 8 cw + (L & 7) and
                // the 16-byte chunks (4 t + (L >> 3) + (L & 7)) mod 32, t = 0..7:
                // conflict-free reads (8 distinct chunk slots per phase) and writes
                // (8 rows of one core matrix).
                const float4 *st = stage + size_t(q) * (kTcTileBytes / 16);
                unsigned char *xh = xbuf + size_t(2 * q) * kTcXBytes, *xl = xh + kTcXBytes;
                const int col = cw * 8 + (lane & 7);
#pragma unroll
                for (int t = 0; t < 8; t++) {
                    const int chunk = (4 * t + (lane >> 3) + (lane & 7)) & 31;  // 4 reals
                    const float4 x = st[col * 32 + chunk];
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
                    *reinterpret_cast<float4 *>(xh + o) = h;
                    *reinterpret_cast<float4 *>(xl + o) = l;
                }
                fence_async_shared();  // the operands are read by the tensor core (async proxy)
                __syncwarp();
                if (lane == 0) mbar_arrive(&bar_x[q]);
            }
            if (j >= 1) {  // tile j - 1 while the tensor core works on tile j
                const uint64_t jp = j - 1;
                const int q = int(jp & 1);
                if (!wait(&bar_mma[q], jp >> 1)) break;
                tc_fence_after();
                float *dst = reinterpret_cast<float *>(tile_ptr(jp));
                const uint32_t taddr = tmem + lane_base + kTcTmemD + uint32_t(q * kTcCols);
                float v[2][16];
#pragma unroll
                for (int h = 0; h < 2; h++) tc_ld16(taddr + uint32_t(half * 32 + h * 16), v[h]);
                tc_wait_ld();
                tc_fence_before();
                __syncwarp();
                if (lane == 0) mbar_arrive(&bar_dfree[q]);
#pragma unroll
                for (int h = 0; h < 2; h++)
#pragma unroll
                    for (int i = 0; i < 16; i++) __stcs(dst + size_t(half * 32 + h * 16 + i) * kTcK + row, v[h][i]);
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (tid == 0 && s_failed) {
        report_timeout(p.err);
        // Copies and MMA batches that may still be in flight (bounded again):
        // only the last two of each, because load j + 2 is issued after tile j
        // was split (so load j had landed) and the MMAs of tile j after D slot
        // j & 1 was read out (so those of tile j - 2 were done).
        for (uint64_t j = loads_issued >= 2 ? loads_issued - 2 : 0; j < loads_issued; j++)
            tc_wait(&bar_load[j & 1], uint32_t((j >> 1) & 1));
        for (uint64_t j = mmas_issued >= 2 ? mmas_issued - 2 : 0; j < mmas_issued; j++)
            tc_wait(&bar_mma[j & 1], uint32_t((j >> 1) & 1));
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
