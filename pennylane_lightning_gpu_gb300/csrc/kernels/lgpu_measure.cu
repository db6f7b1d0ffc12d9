// liblgpu_gb300: measurements.
//
//  * expval of a dense matrix on t bits (FP64 accumulation, deterministic)
//  * Pauli-word expectations: on large states, tile passes that serve up to
//    8 words with different flip masks per read of the state; otherwise one
//    streaming pass per distinct flip mask evaluates up to 16 words through
//    an 8-point Walsh-Hadamard transform of each thread's elements
//  * marginal probabilities: shared-memory histogram per CTA with register
//    run-length accumulation, then a fixed-order cross-CTA sum
//  * sampling: FP64 chunk sums -> single-CTA exclusive scan -> one warp per
//    draw searches its chunk with a warp prefix sum
//  * sum_t c_t P_t |psi> (Hamiltonian apply) and CSR sparse products
#include <cstring>
#include <memory>
#include <type_traits>

#include "lgpu_bodies.cuh"
#include "lgpu_df2.cuh"
#include "lgpu_df64.cuh"
#include "lgpu_internal.cuh"
#include "lgpu_pauli_plan.h"
#include "lgpu_reduce.cuh"

namespace lgpu {

// ---------------------------------------------------------------------------
// Dense matrix expectation in FP64, 4 targets (matrix in the parameter bank;
// 1-3 targets take the float-float kernels below)
// ---------------------------------------------------------------------------
template <class T, class I, int TT> struct ExpvalBody {
    Holes holes;
    I off[1 << TT];
    double m[2 * (1 << TT) * (1 << TT)];
    const cplx_t<T> *sv;
    __device__ __forceinline__ void operator()(I g, double2 *acc) const {
        constexpr int D = 1 << TT;
        const I base = insert_holes<I>(g, holes);
        double ar[D], ai[D];
#pragma unroll
        for (int c = 0; c < D; c++) {
            const cplx_t<T> v = sv[base | off[c]];
            ar[c] = double(v.x);
            ai[c] = double(v.y);
        }
#pragma unroll
        for (int r = 0; r < D; r++) {
            double xr = 0, xi = 0;
#pragma unroll
            for (int c = 0; c < D; c++) {
                const double mr = m[2 * (r * D + c)], mi = m[2 * (r * D + c) + 1];
                xr = fma(mr, ar[c], fma(-mi, ai[c], xr));
                xi = fma(mr, ai[c], fma(mi, ar[c], xi));
            }
            // conj(a_r) * x
            acc[0].x = fma(ar[r], xr, fma(ai[r], xi, acc[0].x));
            acc[0].y = fma(ar[r], xi, fma(-ai[r], xr, acc[0].y));
        }
    }
};

// t = 6..10: one group per CTA iteration, rows split across threads.
template <class T, class I>
__global__ void __launch_bounds__(kReduceBlock)
    expval_big_kernel(const cplx_t<T> *__restrict__ sv, Holes holes, I ngroups, int t, const I *off,
                      const double2 *mat, double2 *partials, unsigned *counter, double2 *out) {
    extern __shared__ double2 stile[];
    __shared__ double2 sm[kReduceBlock / 32];
    const int D = 1 << t;
    double2 acc = make_double2(0.0, 0.0);
    for (I g = blockIdx.x; g < ngroups; g += gridDim.x) {
        const I base = insert_holes<I>(g, holes);
        __syncthreads();
        for (int c = threadIdx.x; c < D; c += kReduceBlock) {
            const cplx_t<T> v = sv[base | off[c]];
            stile[c] = make_double2(double(v.x), double(v.y));
        }
        __syncthreads();
        for (int r = threadIdx.x; r < D; r += kReduceBlock) {
            double xr = 0, xi = 0;
            const double2 *row = mat + size_t(r) * D;
            for (int c = 0; c < D; c++) {
                const double2 mv = row[c], av = stile[c];
                xr = fma(mv.x, av.x, fma(-mv.y, av.y, xr));
                xi = fma(mv.x, av.y, fma(mv.y, av.x, xi));
            }
            const double2 a = stile[r];
            acc.x = fma(a.x, xr, fma(a.y, xi, acc.x));
            acc.y = fma(a.x, xi, fma(-a.y, xr, acc.y));
        }
    }
    __syncthreads();
    double2 v = block_reduce_d2<kReduceBlock>(acc, sm);
    if (threadIdx.x == 0) partials[blockIdx.x] = v;
    if (last_block_arrive(counter)) {
        double2 s = make_double2(0.0, 0.0);
        for (unsigned b = threadIdx.x; b < gridDim.x; b += kReduceBlock) {
            const double2 p = __ldcg(&partials[b]);
            s.x += p.x;
            s.y += p.y;
        }
        __syncthreads();
        s = block_reduce_d2<kReduceBlock>(s, sm);
        if (threadIdx.x == 0) {
            *out = s;
            *counter = 0u;
        }
    }
}

template <class T, class I, int TT>
static lgpu_status_t expval_small(lgpu_context_t ctx, const cplx_t<T> *sv, uint32_t n, const double *matrix,
                                  const std::vector<int> &tg, double *out, int out_on_device, cudaStream_t s) {
    constexpr int D = 1 << TT;
    auto *b = new ExpvalBody<T, I, TT>();
    b->holes = make_holes(tg);
    for (int r = 0; r < D; r++) {
        uint64_t o = 0;
        for (int k = 0; k < TT; k++)
            if ((r >> (TT - 1 - k)) & 1) o |= uint64_t(1) << tg[size_t(k)];
        b->off[r] = I(o);
    }
    std::memcpy(b->m, matrix, sizeof(double) * 2 * D * D);
    b->sv = sv;
    const I ngroups = I(uint64_t(1) << (n - TT));
    const unsigned g = reduce_grid(uint64_t(ngroups));
    ReduceScratch rs;
    lgpu_status_t st = reduce_scratch(ctx, g, 1, &rs);
    if (st != LGPU_OK) {
        delete b;
        return st;
    }
    double2 *res = rs.partials + size_t(g);
    reduce_kernel<1, I><<<g, kReduceBlock, 0, s>>>(*b, ngroups, rs.partials, rs.counter, res);
    delete b;
    LGPU_CHECK_LAUNCH();
    return deliver(ctx, res, 1, out, out_on_device, s);
}

template <class T, class I>
static lgpu_status_t expval_big(lgpu_context_t ctx, const cplx_t<T> *sv, uint32_t n, const double *matrix,
                                const std::vector<int> &tg, double *out, int out_on_device, cudaStream_t s) {
    const int t = int(tg.size());
    const int D = 1 << t;
    std::vector<I> off(static_cast<size_t>(D));
    for (int r = 0; r < D; r++) {
        uint64_t o = 0;
        for (int k = 0; k < t; k++)
            if ((r >> (t - 1 - k)) & 1) o |= uint64_t(1) << tg[size_t(k)];
        off[size_t(r)] = I(o);
    }
    const uint64_t ngroups = uint64_t(1) << (n - t);
    const unsigned g = unsigned(std::min<uint64_t>(ngroups, uint64_t(sm_count()) * 4));
    const size_t mbytes = size_t(D) * D * sizeof(double2);
    const size_t obytes = size_t(D) * sizeof(I);
    void *p = nullptr;
    const size_t head = 256 + size_t(g) * sizeof(double2) + 256;
    LGPU_TRY(ctx_scratch(ctx, head + mbytes + obytes + 256, &p));
    auto *counter = static_cast<unsigned *>(p);
    auto *partials = reinterpret_cast<double2 *>(static_cast<char *>(p) + 256);
    auto *res = partials + g;
    auto *dmat = reinterpret_cast<double2 *>(static_cast<char *>(p) + head);
    auto *doff = reinterpret_cast<I *>(static_cast<char *>(p) + head + mbytes);
    LGPU_CUDA_TRY(cudaMemcpyAsync(dmat, matrix, mbytes, cudaMemcpyHostToDevice, s));
    LGPU_CUDA_TRY(cudaMemcpyAsync(doff, off.data(), obytes, cudaMemcpyHostToDevice, s));
    const size_t smem = size_t(D) * sizeof(double2);
    static std::atomic<size_t> attr_e[64];
    LGPU_TRY(ensure_smem(reinterpret_cast<const void *>(expval_big_kernel<T, I>), smem, attr_e));
    expval_big_kernel<T, I><<<g, kReduceBlock, smem, s>>>(sv, make_holes(tg), I(ngroups), t, doff, dmat, partials,
                                                         counter, res);
    LGPU_CHECK_LAUNCH();
    return deliver(ctx, res, 1, out, out_on_device, s);
}

// ---------------------------------------------------------------------------
// Dense matrix expectation on t = 11..13 targets (a Hamiltonian of up to 13
// wires handed over as one dense matrix of 2^t x 2^t, up to 1 GiB).  Work
// items are (group g, chunk of kGemvRows rows); each CTA takes a contiguous
// range of items, copies its group's 2^t amplitudes into shared memory as
// double2 (reloaded only when the group changes) and each warp forms, for
// its kGemvRows / 8 rows, x_r = sum_c M_rc a_c with the lanes striding the
// row (coalesced reads of the row-major matrix, a fixed order per lane and a
// fixed shuffle tree), then conj(a_r) x_r.  FP64 throughout; deterministic.
// ---------------------------------------------------------------------------
constexpr int kGemvRows = 32;

template <class T, class I>
__global__ void __launch_bounds__(kReduceBlock)
    expval_gemv_kernel(const cplx_t<T> *__restrict__ sv, Holes holes, uint64_t nitems, uint64_t per_cta, int t,
                       const I *__restrict__ off, const double2 *__restrict__ mat, double2 *partials,
                       unsigned *counter, double2 *out) {
    extern __shared__ double2 stile[];
    __shared__ double2 sm[kReduceBlock / 32];
    const int D = 1 << t;
    const int chunks_log = t - 5;  // log2(D / kGemvRows)
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    constexpr int kRowsPerWarp = kGemvRows / (kReduceBlock / 32);
    double2 acc = make_double2(0.0, 0.0);
    const uint64_t first = uint64_t(blockIdx.x) * per_cta;
    const uint64_t last = first + per_cta < nitems ? first + per_cta : nitems;
    I loaded = ~I(0);
    for (uint64_t item = first; item < last; item++) {
        const I g = I(item >> chunks_log);
        const int chunk = int(item & ((uint64_t(1) << chunks_log) - 1));
        if (g != loaded) {
            const I base = insert_holes<I>(g, holes);
            __syncthreads();
            for (int c = threadIdx.x; c < D; c += kReduceBlock) {
                const cplx_t<T> v = sv[base | off[c]];
                stile[c] = make_double2(double(v.x), double(v.y));
            }
            __syncthreads();
            loaded = g;
        }
#pragma unroll 1
        for (int rr = 0; rr < kRowsPerWarp; rr++) {
            const int r = chunk * kGemvRows + warp * kRowsPerWarp + rr;
            const double2 *row = mat + size_t(r) * size_t(D);
            double xr = 0.0, xi = 0.0;
            for (int c = lane; c < D; c += 32) {
                const double2 mv = __ldg(&row[c]), av = stile[c];
                xr = fma(mv.x, av.x, fma(-mv.y, av.y, xr));
                xi = fma(mv.x, av.y, fma(mv.y, av.x, xi));
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                xr += __shfl_xor_sync(0xffffffffu, xr, o);
                xi += __shfl_xor_sync(0xffffffffu, xi, o);
            }
            if (lane == 0) {
                const double2 a = stile[r];
                acc.x = fma(a.x, xr, fma(a.y, xi, acc.x));
                acc.y = fma(a.x, xi, fma(-a.y, xr, acc.y));
            }
        }
    }
    __syncthreads();
    double2 v = block_reduce_d2<kReduceBlock>(acc, sm);
    if (threadIdx.x == 0) partials[blockIdx.x] = v;
    if (last_block_arrive(counter)) {
        double2 s = make_double2(0.0, 0.0);
        for (unsigned b = threadIdx.x; b < gridDim.x; b += kReduceBlock) {
            const double2 p = __ldcg(&partials[b]);
            s.x += p.x;
            s.y += p.y;
        }
        __syncthreads();
        s = block_reduce_d2<kReduceBlock>(s, sm);
        if (threadIdx.x == 0) {
            *out = s;
            *counter = 0u;
        }
    }
}

template <class T, class I>
static lgpu_status_t expval_gemv(lgpu_context_t ctx, const cplx_t<T> *sv, uint32_t n, const double *matrix,
                                 const std::vector<int> &tg, double *out, int out_on_device, cudaStream_t s) {
    const int t = int(tg.size());
    const int D = 1 << t;
    std::vector<I> off(static_cast<size_t>(D));
    for (int r = 0; r < D; r++) {
        uint64_t o = 0;
        for (int k = 0; k < t; k++)
            if ((r >> (t - 1 - k)) & 1) o |= uint64_t(1) << tg[size_t(k)];
        off[size_t(r)] = I(o);
    }
    const uint64_t ngroups = uint64_t(1) << (n - t);
    const uint64_t nitems = ngroups << (t - 5);
    const size_t smem = size_t(D) * sizeof(double2);
    // resident CTAs per SM at this shared-memory size (227 KB usable per SM)
    const unsigned per_sm = unsigned(std::max<size_t>(1, std::min<size_t>(4, (size_t(227) << 10) / (smem + 2048))));
    const unsigned g = unsigned(std::min<uint64_t>(nitems, uint64_t(sm_count()) * per_sm));
    const uint64_t per_cta = (nitems + g - 1) / g;
    const size_t mbytes = size_t(D) * D * sizeof(double2);
    const size_t obytes = size_t(D) * sizeof(I);
    void *p = nullptr;
    const size_t head = 256 + size_t(g) * sizeof(double2) + 256;
    LGPU_TRY(ctx_scratch(ctx, head + mbytes + obytes + 256, &p));
    auto *counter = static_cast<unsigned *>(p);
    auto *partials = reinterpret_cast<double2 *>(static_cast<char *>(p) + 256);
    auto *res = partials + g;
    auto *dmat = reinterpret_cast<double2 *>(static_cast<char *>(p) + head);
    auto *doff = reinterpret_cast<I *>(static_cast<char *>(p) + head + mbytes);
    LGPU_CUDA_TRY(cudaMemcpyAsync(dmat, matrix, mbytes, cudaMemcpyHostToDevice, s));
    LGPU_CUDA_TRY(cudaMemcpyAsync(doff, off.data(), obytes, cudaMemcpyHostToDevice, s));
    static std::atomic<size_t> attr_g[64];
    LGPU_TRY(ensure_smem(reinterpret_cast<const void *>(expval_gemv_kernel<T, I>), smem, attr_g));
    expval_gemv_kernel<T, I><<<g, kReduceBlock, smem, s>>>(sv, make_holes(tg), nitems, per_cta, t, doff, dmat,
                                                          partials, counter, res);
    LGPU_CHECK_LAUNCH();
    return deliver(ctx, res, 1, out, out_on_device, s);
}

// ---------------------------------------------------------------------------
// Dense matrix expectation, t <= 2, without FP64 work per amplitude:
// <a|M|a> = sum_rc M_rc G_rc with the Gram sums G_rc = sum_g conj(a_gr) a_gc
// (Hermitian: D real diagonal sums and D(D-1)/2 complex ones).  Each thread
// forms the products in float-float (complex128 amplitudes are split first),
// sums 16 runs of UB groups in float-float, then adds them to a double; the
// last CTA contracts the reduced G with M in double.
// ---------------------------------------------------------------------------
template <class T, class I, int TT> struct GramParams {
    Holes holes;
    I off[1 << TT];
    I ngroups;
    double m[2 * (1 << TT) * (1 << TT)];
    const cplx_t<T> *sv;
};

__device__ __forceinline__ DF to_df(float x) { return DF{x, 0.0f}; }
__device__ __forceinline__ DF to_df(double x) { return df_from_double(x); }

template <class T, class I, int TT>
__global__ void __launch_bounds__(kReduceBlock)
    gram_expval_kernel(const GramParams<T, I, TT> p, double2 *partials, unsigned *counter, double2 *out) {
    constexpr int D = 1 << TT, NA = D * D, N2 = NA / 2, UB = TT == 1 ? 4 : 2;
    __shared__ double2 sm[kReduceBlock / 32];
    __shared__ double gsum[NA];
    double accd[NA];
#pragma unroll
    for (int j = 0; j < NA; j++) accd[j] = 0.0;
    const I stride = I(gridDim.x) * kReduceBlock;
    DF acc[NA];
#pragma unroll
    for (int j = 0; j < NA; j++) acc[j] = DF{0.0f, 0.0f};
    int runs = 0;
    for (I g0 = I(blockIdx.x) * kReduceBlock + threadIdx.x; g0 < p.ngroups; g0 += I(UB) * stride) {
        cplx_t<T> v[UB][D];
#pragma unroll
        for (int u = 0; u < UB; u++) {
            const I g = g0 + I(u) * stride;
            const bool ok = g < p.ngroups;
            const I base = insert_holes<I>(ok ? g : I(0), p.holes);
#pragma unroll
            for (int c = 0; c < D; c++) v[u][c] = ok ? p.sv[base | p.off[c]] : cplx_t<T>{};
        }
#pragma unroll
        for (int u = 0; u < UB; u++) {
            DF ar[D], ai[D];
#pragma unroll
            for (int c = 0; c < D; c++) {
                ar[c] = to_df(v[u][c].x);
                ai[c] = to_df(v[u][c].y);
            }
#pragma unroll
            for (int r = 0; r < D; r++) acc[r] = df_sum<3>({acc[r], df_mul(ar[r], ar[r]), df_mul(ai[r], ai[r])});
            int k = D;
#pragma unroll
            for (int r = 0; r < D; r++)
#pragma unroll
                for (int c = r + 1; c < D; c++) {
                    acc[k] = df_sum<3>({acc[k], df_mul(ar[r], ar[c]), df_mul(ai[r], ai[c])});
                    acc[k + 1] = df_sum<3>({acc[k + 1], df_mul(ar[r], ai[c]), df_neg(df_mul(ai[r], ar[c]))});
                    k += 2;
                }
        }
        if (++runs == 16) {  // 16 runs of UB groups in float-float, then into the doubles
            runs = 0;
#pragma unroll
            for (int j = 0; j < NA; j++) {
                accd[j] += df_to_double(acc[j]);
                acc[j] = DF{0.0f, 0.0f};
            }
        }
    }
#pragma unroll
    for (int j = 0; j < NA; j++) accd[j] += df_to_double(acc[j]);
#pragma unroll
    for (int k = 0; k < N2; k++) {
        const double2 v = block_reduce_d2<kReduceBlock>(make_double2(accd[2 * k], accd[2 * k + 1]), sm);
        if (threadIdx.x == 0) partials[size_t(blockIdx.x) * N2 + k] = v;
        __syncthreads();
    }
    if (last_block_arrive(counter)) {
#pragma unroll
        for (int k = 0; k < N2; k++) {
            double2 s = make_double2(0.0, 0.0);
            for (unsigned b = threadIdx.x; b < gridDim.x; b += kReduceBlock) {
                const double2 q = __ldcg(&partials[size_t(b) * N2 + k]);
                s.x += q.x;
                s.y += q.y;
            }
            s = block_reduce_d2<kReduceBlock>(s, sm);
            if (threadIdx.x == 0) {
                gsum[2 * k] = s.x;
                gsum[2 * k + 1] = s.y;
            }
            __syncthreads();
        }
        if (threadIdx.x == 0) {
            double re = 0.0, im = 0.0;
            for (int r = 0; r < D; r++) {  // M_rr G_rr
                re += p.m[2 * (r * D + r)] * gsum[r];
                im += p.m[2 * (r * D + r) + 1] * gsum[r];
            }
            int k = D;
            for (int r = 0; r < D; r++)
                for (int c = r + 1; c < D; c++) {  // M_rc G_rc + M_cr conj(G_rc)
                    const double gr = gsum[k], gi = gsum[k + 1];
                    const double ar = p.m[2 * (r * D + c)], ai = p.m[2 * (r * D + c) + 1];
                    const double br = p.m[2 * (c * D + r)], bi = p.m[2 * (c * D + r) + 1];
                    re += ar * gr - ai * gi + br * gr + bi * gi;
                    im += ar * gi + ai * gr + bi * gr - br * gi;
                    k += 2;
                }
            *out = make_double2(re, im);
            *counter = 0u;
        }
    }
}

template <class T, class I, int TT>
static lgpu_status_t expval_gram(lgpu_context_t ctx, const cplx_t<T> *sv, uint32_t n, const double *matrix,
                                 const std::vector<int> &tg, double *out, int out_on_device, cudaStream_t s) {
    constexpr int D = 1 << TT, N2 = D * D / 2;
    GramParams<T, I, TT> p{};
    p.holes = make_holes(tg);
    for (int r = 0; r < D; r++) {
        uint64_t o = 0;
        for (int k = 0; k < TT; k++)
            if ((r >> (TT - 1 - k)) & 1) o |= uint64_t(1) << tg[size_t(k)];
        p.off[r] = I(o);
    }
    p.ngroups = I(uint64_t(1) << (n - TT));
    std::memcpy(p.m, matrix, sizeof(double) * 2 * D * D);
    p.sv = sv;
    const unsigned g = reduce_grid(uint64_t(p.ngroups));
    ReduceScratch rs;
    LGPU_TRY(reduce_scratch(ctx, g, N2, &rs));
    double2 *res = rs.partials + size_t(g) * N2;
    gram_expval_kernel<T, I, TT><<<g, kReduceBlock, 0, s>>>(p, rs.partials, rs.counter, res);
    LGPU_CHECK_LAUNCH();
    return deliver(ctx, res, 1, out, out_on_device, s);
}

// Dense matrix expectation on 3 targets in float-float: per group of 8
// amplitudes conj(a) . (M a) (df_expval_group), 16 groups per thread summed
// in float-float before each double flush, fixed-order reduction.
template <class T, class I, int TT> struct DfExpvalParams {
    Holes holes;
    I off[1 << TT];
    I ngroups;
    DF m[2 * (1 << TT) * (1 << TT)];  // (re, im) of M_rc, row-major
    const cplx_t<T> *sv;
};

template <class T, class I, int TT>
__global__ void __launch_bounds__(kReduceBlock)
    expval_df_kernel(const __grid_constant__ DfExpvalParams<T, I, TT> p, double2 *partials, unsigned *counter,
                     double2 *out) {
    constexpr int D = 1 << TT;
    __shared__ double2 sm[kReduceBlock / 32];
    double2 accd = make_double2(0.0, 0.0);
    DF re{0.0f, 0.0f}, im{0.0f, 0.0f};
    int runs = 0;
    const I stride = I(gridDim.x) * kReduceBlock;
    for (I g = I(blockIdx.x) * kReduceBlock + threadIdx.x; g < p.ngroups; g += stride) {
        const I base = insert_holes<I>(g, p.holes);
        DF ar[D], ai[D];
#pragma unroll
        for (int c = 0; c < D; c++) {
            const cplx_t<T> v = p.sv[base | p.off[c]];
            ar[c] = to_df(v.x);
            ai[c] = to_df(v.y);
        }
        df_expval_group<D>(p.m, ar, ai, re, im);
        if (++runs == 16) {
            runs = 0;
            accd.x += df_to_double(re);
            accd.y += df_to_double(im);
            re = DF{0.0f, 0.0f};
            im = DF{0.0f, 0.0f};
        }
    }
    accd.x += df_to_double(re);
    accd.y += df_to_double(im);
    const double2 v = block_reduce_d2<kReduceBlock>(accd, sm);
    if (threadIdx.x == 0) partials[blockIdx.x] = v;
    __syncthreads();
    if (last_block_arrive(counter)) {
        double2 t = make_double2(0.0, 0.0);
        for (unsigned b = threadIdx.x; b < gridDim.x; b += kReduceBlock) {
            const double2 q = __ldcg(&partials[b]);
            t.x += q.x;
            t.y += q.y;
        }
        t = block_reduce_d2<kReduceBlock>(t, sm);
        if (threadIdx.x == 0) {
            *out = t;
            *counter = 0u;
        }
    }
}

template <class T, class I, int TT>
static lgpu_status_t expval_df(lgpu_context_t ctx, const cplx_t<T> *sv, uint32_t n, const double *matrix,
                               const std::vector<int> &tg, double *out, int out_on_device, cudaStream_t s) {
    constexpr int D = 1 << TT;
    auto *p = new DfExpvalParams<T, I, TT>();
    p->holes = make_holes(tg);
    for (int r = 0; r < D; r++) {
        uint64_t o = 0;
        for (int k = 0; k < TT; k++)
            if ((r >> (TT - 1 - k)) & 1) o |= uint64_t(1) << tg[size_t(k)];
        p->off[r] = I(o);
    }
    p->ngroups = I(uint64_t(1) << (n - TT));
    for (int i = 0; i < 2 * D * D; i++) p->m[i] = df_split_host(matrix[i]);
    p->sv = sv;
    const unsigned g = reduce_grid(uint64_t(p->ngroups));
    ReduceScratch rs;
    lgpu_status_t st = reduce_scratch(ctx, g, 1, &rs);
    if (st != LGPU_OK) {
        delete p;
        return st;
    }
    double2 *res = rs.partials + size_t(g);
    expval_df_kernel<T, I, TT><<<g, kReduceBlock, 0, s>>>(*p, rs.partials, rs.counter, res);
    delete p;
    LGPU_CHECK_LAUNCH();
    return deliver(ctx, res, 1, out, out_on_device, s);
}

template <class T, class I>
static lgpu_status_t expval_dispatch(lgpu_context_t ctx, const void *sv, uint32_t n, const double *matrix,
                                     const std::vector<int> &tg, double *out, int od, cudaStream_t s) {
    const auto *p = static_cast<const cplx_t<T> *>(sv);
    switch (tg.size()) {
    case 1: return expval_gram<T, I, 1>(ctx, p, n, matrix, tg, out, od, s);
    case 2: return expval_gram<T, I, 2>(ctx, p, n, matrix, tg, out, od, s);
    case 3: return expval_df<T, I, 3>(ctx, p, n, matrix, tg, out, od, s);
    case 4: return expval_small<T, I, 4>(ctx, p, n, matrix, tg, out, od, s);
    default:
        if (tg.size() > 10) return expval_gemv<T, I>(ctx, p, n, matrix, tg, out, od, s);
        return expval_big<T, I>(ctx, p, n, matrix, tg, out, od, s);
    }
}

// ---------------------------------------------------------------------------
// Pauli words
// ---------------------------------------------------------------------------
constexpr int kWordsPerPass = 8;

template <class T, class I> struct PauliBody {
    const cplx_t<T> *sv;
    Holes holes;   // lowest flip bit (empty when flip == 0)
    I flip;
    int nt;
    I sgn[kWordsPerPass];
    int kappa_neg[kWordsPerPass];  // parity(flip & sgn) odd
    __device__ __forceinline__ void operator()(I g, double2 *acc) const {
        if (flip == 0) {
            const I i = g;
            const cplx_t<T> a = sv[i];
            const double p = fma(double(a.x), double(a.x), double(a.y) * double(a.y));
#pragma unroll
            for (int t = 0; t < kWordsPerPass; t++) {
                if (t < nt) acc[t].x += (__popcll(uint64_t(i & sgn[t])) & 1) ? -p : p;
            }
        } else {
            const I i = insert_holes<I>(g, holes);
            const I j = i ^ flip;
            const cplx_t<T> a = sv[i], b = sv[j];
            // w = conj(a) b
            const double wr = fma(double(a.x), double(b.x), double(a.y) * double(b.y));
            const double wi = fma(double(a.x), double(b.y), -double(a.y) * double(b.x));
#pragma unroll
            for (int t = 0; t < kWordsPerPass; t++) {
                if (t < nt) {
                    const double sg = (__popcll(uint64_t(i & sgn[t])) & 1) ? -2.0 : 2.0;
                    if (kappa_neg[t])
                        acc[t].y -= sg * wi;
                    else
                        acc[t].x += sg * wr;
                }
            }
        }
    }
};

// Walsh-Hadamard form of the Pauli-word pass (states of >= 4 qubits).  The
// items of a pass (all indices, or the indices with the lowest flip bit clear)
// are split as item = slot + S*j, j = 0..7 in the top three item bits.  A
// thread loads the eight elements of a slot, forms w_j = conj(a) a^flip (or
// |a|^2), and takes the 8-point transform W[h] = sum_j (-1)^popc(j & h) w_j.
// A word with sign mask s then adds (-1)^popc(base & s) W[h_s], h_s the bits
// of s under the three j bits: per word one popcount, one select and one add
// per eight elements, instead of a signed FP64 add per element.  complex64
// transforms in FP32 and flushes chunks of 16 slots into FP64 accumulators.
constexpr int kWhtWords = 16;

template <class T, class I> struct PauliWhtParams {
    const cplx_t<T> *sv;
    Holes holes;  // lowest flip bit (none when flip == 0)
    I flip;
    I slots;      // items / 8
    int lgS;
    int nt;
    uint32_t use_im;  // bit t: word t reads the imaginary transform
    int need_re, need_im;  // some word of the pass reads the real / imaginary products
    int direct;            // few words: each word's one coefficient as a signed 8-term sum
    I sgn[kWhtWords];
    uint32_t hsel[kWhtWords];
};

__device__ __forceinline__ void wht_cp_async(void *smem_dst, const void *gsrc, int bytes) {
    const uint32_t d = static_cast<uint32_t>(__cvta_generic_to_shared(smem_dst));
    if (bytes == 16)
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(gsrc) : "memory");
    else
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(d), "l"(gsrc) : "memory");
}

// Each thread streams its slots through a private two-stage ring in shared
// memory ([stage][a|b][j][thread]): the next slot's loads are in flight while
// the current slot is transformed (no barrier: a thread reads only its own
// copies, after cp.async.wait_group).
constexpr int kDirectWords = 3;

// NEED (1 real, 2 imaginary, 3 both) selects the products at compile time.
template <class T, class I, bool DIRECT, int NEED>
__global__ void __launch_bounds__(kReduceBlock, 2)
    pauli_wht_kernel(const PauliWhtParams<T, I> p, double2 *partials, unsigned *counter, double2 *out) {
    using C = cplx_t<T>;
    constexpr bool kChunk = sizeof(T) == 4;
    extern __shared__ __align__(16) unsigned char wht_smem[];
    C *ring = reinterpret_cast<C *>(wht_smem);  // [2][2][8][kReduceBlock]
    auto at = [&](int st, int ab, int j) -> C * { return ring + ((st * 2 + ab) * 8 + j) * kReduceBlock + threadIdx.x; };
    __shared__ double2 sm[kReduceBlock / 32];
    double acc[kWhtWords];
    T chunk[kWhtWords];
#pragma unroll
    for (int t = 0; t < kWhtWords; t++) {
        acc[t] = 0.0;
        chunk[t] = T(0);
    }
    I off[8];
#pragma unroll
    for (int j = 0; j < 8; j++) off[j] = insert_holes<I>(I(j) << p.lgS, p.holes);
    auto prefetch = [&](I slot, int st) {
        const I base = insert_holes<I>(slot, p.holes);
#pragma unroll
        for (int j = 0; j < 8; j++) {
            wht_cp_async(at(st, 0, j), &p.sv[base | off[j]], int(sizeof(C)));
            if (p.flip) wht_cp_async(at(st, 1, j), &p.sv[(base | off[j]) ^ p.flip], int(sizeof(C)));
        }
        asm volatile("cp.async.commit_group;" ::: "memory");
    };
    int cn = 0;
    const I stride = I(gridDim.x) * kReduceBlock;
    I slot = I(blockIdx.x) * kReduceBlock + threadIdx.x;
    if (slot < p.slots) prefetch(slot, 0);
    else asm volatile("cp.async.commit_group;" ::: "memory");
    for (int it = 0; slot < p.slots; slot += stride, it++) {
        const int st = it & 1;
        if (slot + stride < p.slots) prefetch(slot + stride, st ^ 1);
        else asm volatile("cp.async.commit_group;" ::: "memory");
        asm volatile("cp.async.wait_group 1;" ::: "memory");
        const I base = insert_holes<I>(slot, p.holes);
        T wr[8], wi[8];
        if (p.flip) {
#pragma unroll
            for (int j = 0; j < 8; j++) {
                const C a = *at(st, 0, j), b = *at(st, 1, j);
                if constexpr ((NEED & 1) != 0) wr[j] = a.x * b.x + a.y * b.y;
                else wr[j] = T(0);
                if constexpr ((NEED & 2) != 0) wi[j] = a.x * b.y - a.y * b.x;
                else wi[j] = T(0);
            }
        } else {
#pragma unroll
            for (int j = 0; j < 8; j++) {
                const C a = *at(st, 0, j);
                wr[j] = a.x * a.x + a.y * a.y;
                wi[j] = T(0);
            }
        }
        if constexpr (!DIRECT) {
            if constexpr ((NEED & 1) != 0) wht8(wr);
            if constexpr ((NEED & 2) != 0) wht8(wi);
        }
#pragma unroll
        for (int t = 0; t < (DIRECT ? kDirectWords : kWhtWords); t++) {
            if (t < p.nt) {
                const bool im = (p.use_im >> t) & 1u;
                T v;
                if constexpr (DIRECT) {
                    // W[h] = sum_j (-1)^popc(j & h) x_j for this word's h only
                    const uint32_t h = p.hsel[t];
                    v = T(0);
#pragma unroll
                    for (int j = 0; j < 8; j++) {
                        const T x = im ? wi[j] : wr[j];
                        v += (__popc(uint32_t(j) & h) & 1) ? -x : x;
                    }
                } else {
                    v = im ? sel8(wi, p.hsel[t]) : sel8(wr, p.hsel[t]);
                }
                const T c = (__popcll(uint64_t(base & p.sgn[t])) & 1) ? -v : v;
                if constexpr (kChunk)
                    chunk[t] += c;
                else
                    acc[t] += c;
            }
        }
        if constexpr (kChunk) {
            if (++cn == 16) {
#pragma unroll
                for (int t = 0; t < kWhtWords; t++) {
                    acc[t] += double(chunk[t]);
                    chunk[t] = T(0);
                }
                cn = 0;
            }
        }
    }
    asm volatile("cp.async.wait_group 0;" ::: "memory");
    if constexpr (kChunk) {
#pragma unroll
        for (int t = 0; t < kWhtWords; t++) acc[t] += double(chunk[t]);
    }
#pragma unroll
    for (int t = 0; t < kWhtWords; t++) {
        const double2 v = block_reduce_d2<kReduceBlock>(make_double2(acc[t], 0.0), sm);
        if (threadIdx.x == 0) partials[size_t(blockIdx.x) * kWhtWords + t] = v;
        __syncthreads();
    }
    if (last_block_arrive(counter)) {
#pragma unroll 1
        for (int t = 0; t < kWhtWords; t++) {
            double2 s = make_double2(0.0, 0.0);
            for (unsigned b = threadIdx.x; b < gridDim.x; b += kReduceBlock) {
                const double2 q = __ldcg(&partials[size_t(b) * kWhtWords + t]);
                s.x += q.x;
            }
            s = block_reduce_d2<kReduceBlock>(s, sm);
            if (threadIdx.x == 0) out[t] = s;
            __syncthreads();
        }
        if (threadIdx.x == 0) *counter = 0u;
    }
}

template <class T> constexpr size_t wht_smem_bytes() { return size_t(2) * 2 * 8 * kReduceBlock * sizeof(cplx_t<T>); }

// Launch one pass with the compile-time product selection (opts the
// instantiation in to its shared memory first).
template <class T, class I, bool DIRECT, int NEED>
static lgpu_status_t wht_launch(const PauliWhtParams<T, I> &b, unsigned g, double2 *partials, unsigned *counter,
                                double2 *out, cudaStream_t s) {
    static std::atomic<size_t> attr[64];
    LGPU_TRY(ensure_smem(reinterpret_cast<const void *>(pauli_wht_kernel<T, I, DIRECT, NEED>), wht_smem_bytes<T>(),
                         attr));
    pauli_wht_kernel<T, I, DIRECT, NEED><<<g, kReduceBlock, wht_smem_bytes<T>(), s>>>(b, partials, counter, out);
    LGPU_CHECK_LAUNCH();
    return LGPU_OK;
}

template <class T, class I, bool DIRECT>
static lgpu_status_t wht_dispatch(const PauliWhtParams<T, I> &b, unsigned g, double2 *partials, unsigned *counter,
                                  double2 *out, cudaStream_t s) {
    const int need = (b.need_re ? 1 : 0) | (b.need_im ? 2 : 0);
    switch (need) {
    case 2: return wht_launch<T, I, DIRECT, 2>(b, g, partials, counter, out, s);
    case 3: return wht_launch<T, I, DIRECT, 3>(b, g, partials, counter, out, s);
    default: return wht_launch<T, I, DIRECT, 1>(b, g, partials, counter, out, s);
    }
}

// ---------------------------------------------------------------------------
// Tiled Pauli-word passes: words with different flip masks in one read.
// A tile is 2^K amplitudes (K = 12 for complex64, 11 for complex128: 32 KB):
// the low run 0..m-1 of state bits (runs of at least 128 bytes) plus up to
// kTileHiMax higher bits.  Every word of a pass flips only tile bits, so each
// pair (x, x ^ flip) lies in one tile.  A CTA streams tiles through two
// shared-memory buffers (cp.async); complex128 tiles are converted after the
// load to float-float, (re.hi, im.hi, re.lo, im.lo) per amplitude.
//
// The work of a thread has a fixed shape.  Tile element e = tid + 256 j (tid
// the thread, j = 0 .. E/256 - 1): the sign (-1)^popc(e & sign) of a diagonal
// word splits into a per-thread bit and a per-word constant bit for j, and
// |a_e|^2 is formed once per element for all diagonal words of the pass.  For
// a word with flips, pair c = tid + 256 j has its first element x = c with a
// zero inserted at the lowest flip position b0, so x = X | J_j with X from the
// thread and J_j from j on disjoint bits; its partner x ^ flip =
// (X ^ (flip off the J bits)) | (J_j ^ (flip on the J bits)), again disjoint.
// Both addresses are a per-thread base plus a per-word constant, and the sign
// a per-thread bit XOR a per-word constant bit: no index walk and no
// population count per pair.
//
// Sums: complex64 in float per thread (each thread's share is small);
// complex128 in float-float, products split exactly by FMA and two running
// sums per word (even and odd j), so the TwoSum chains of neighbouring pairs
// overlap.  At the end warp sums go to per-warp double slots; a CTA writes its
// totals and a second kernel sums the CTAs in a fixed order.  The raw sums
// equal those of the Walsh-Hadamard pass.
// ---------------------------------------------------------------------------
constexpr int kPauliTileThreads = 256;

template <class T> struct PtGeom {
    static constexpr int K = sizeof(T) == 4 ? 12 : 11;   // tile bits (32 KB tiles)
    static constexpr int E = 1 << K;                     // elements per tile
    static constexpr int NA = E / kPauliTileThreads;     // elements per thread
    static constexpr int NP = NA / 2;                    // pairs per thread and word
    static constexpr int LEB = sizeof(T) == 4 ? 3 : 4;   // log2 of the bytes per tile element
    static constexpr int MMIN = sizeof(T) == 4 ? 4 : 3;  // runs of at least 128 bytes
};
constexpr int kPtMaxNA = 16;
static_assert(PtGeom<float>::NA <= kPtMaxNA && PtGeom<double>::NA <= kPtMaxNA, "per-thread element count");
static_assert((kPauliTileThreads & (kPauliTileThreads - 1)) == 0 && kPauliTileThreads == 256,
              "the j part of a tile index starts at bit 8");

template <class I> struct PauliTileParams {
    const void *sv;
    Holes holes;  // tile bit positions
    I ntiles;
    int m, nw, nd;                          // low run; words; the first nd are diagonal
    uint32_t use_im;                        // bit t: word t sums Im(conj(a_x) a_{x^flip})
    I hi_off[1 << kTileHiMax];              // state offset of each run of 2^m amplitudes
    uint32_t tsign[kTileWords];             // sign mask in tile positions
    uint64_t osign[kTileWords];             // sign mask outside the tile (state bits)
    uint32_t b0[kTileWords];                // words with flips: lowest flip position
    uint32_t fxb[kTileWords];               // flip bits off the J bits, times the element bytes
    uint32_t ja[kTileWords][kPtMaxNA / 2];  // J_j times the element bytes
    uint32_t jb[kTileWords][kPtMaxNA / 2];  // (J_j ^ flip bits on the J bits) times the element bytes
    uint32_t cs[kTileWords][kPtMaxNA];      // bit 31: parity of (the j part & the sign mask)
    double *partials;                       // [gridDim.x][nw]
};

template <class T> struct TileAcc;
template <> struct TileAcc<float> {
    float v = 0.0f;
    __device__ __forceinline__ void warp_reduce() {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    }
    __device__ __forceinline__ double value() const { return double(v); }
};
template <> struct TileAcc<double> {
    DF2 v{F2{0ull}, F2{0ull}};  // two running sums in the lanes, unnormalised
    DF r{0.0f, 0.0f};
    __device__ __forceinline__ void warp_reduce() {
        DF s = df_sum<2>({DF{f2_x(v.hi), f2_x(v.lo)}, DF{f2_y(v.hi), f2_y(v.lo)}});  // renormalised
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            s = df_sum<2>({s, DF{__shfl_xor_sync(0xffffffffu, s.hi, o), __shfl_xor_sync(0xffffffffu, s.lo, o)}});
        r = s;
    }
    __device__ __forceinline__ double value() const { return df_to_double(r); }
};

// a with the sign bits sx, sy XOR-ed into its lanes.
__device__ __forceinline__ F2 f2_flip(F2 a, uint32_t sx, uint32_t sy) {
    return f2_pack(__uint_as_float(__float_as_uint(f2_x(a)) ^ sx), __uint_as_float(__float_as_uint(f2_y(a)) ^ sy));
}

// acc += (sx a_x b_x, sy a_y b_y) lane by lane for float-float lanes a, b and
// signs given as the bit patterns 0 / 0x80000000.  The leading products are
// split exactly (a scalar FMA per lane for the error, which negates an
// operand for free), the sums by TwoSum; the error terms and the cross
// products gather in acc.lo, which stays unnormalised until the end.
__device__ __forceinline__ void df2_acc_mul(DF2 &acc, uint32_t sx, uint32_t sy, const DF2 &a, const DF2 &b) {
    F2 p = f2_mul(a.hi, b.hi);
    const float ex = __fmaf_rn(f2_x(a.hi), f2_x(b.hi), -f2_x(p));
    const float ey = __fmaf_rn(f2_y(a.hi), f2_y(b.hi), -f2_y(p));
    F2 e = f2_fma(a.hi, b.lo, f2_pack(ex, ey));
    e = f2_fma(a.lo, b.hi, e);
    p = f2_flip(p, sx, sy);
    e = f2_flip(e, sx, sy);
    const F2 h = f2_add(acc.hi, p);
    const F2 bb = f2_sub(h, acc.hi);
    const F2 err = f2_add(f2_sub(acc.hi, f2_sub(h, bb)), f2_sub(p, bb));
    acc.lo = f2_add(acc.lo, f2_add(err, e));
    acc.hi = h;
}

// acc += (sx q_x, sy q_y) lane by lane for unnormalised float-float lanes q.
__device__ __forceinline__ void df2_acc_signed(DF2 &acc, uint32_t sx, uint32_t sy, F2 qh, F2 ql) {
    qh = f2_flip(qh, sx, sy);
    ql = f2_flip(ql, sx, sy);
    const F2 h = f2_add(acc.hi, qh);
    const F2 bb = f2_sub(h, acc.hi);
    const F2 err = f2_add(f2_sub(acc.hi, f2_sub(h, bb)), f2_sub(qh, bb));
    acc.lo = f2_add(acc.lo, f2_add(err, ql));
    acc.hi = h;
}

__device__ __forceinline__ float pt_flip_sign(float x, uint32_t sbit) { return __uint_as_float(__float_as_uint(x) ^ sbit); }

__device__ __forceinline__ void pt_cp_async16(void *smem_dst, const void *gsrc) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(static_cast<uint32_t>(__cvta_generic_to_shared(smem_dst))),
                 "l"(gsrc)
                 : "memory");
}

__device__ __forceinline__ uint32_t pt_insert_zero(uint32_t v, uint32_t b) {
    const uint32_t low = (1u << b) - 1u;
    return ((v & ~low) << 1) | (v & low);
}

// A float-float copy of a complex128 state, (re.hi, im.hi, re.lo, im.lo) per
// amplitude: tile passes over it skip the per-tile conversion.
__global__ void __launch_bounds__(256) df_state_copy_kernel(const double2 *__restrict__ src, float4 *__restrict__ dst,
                                                             uint64_t count) {
    const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
    for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < count; i += stride) {
        const double2 v = src[i];
        const DF r = df_from_double(v.x), im = df_from_double(v.y);
        dst[i] = make_float4(r.hi, im.hi, r.lo, im.lo);
    }
}

// DFSRC: the complex128 source is already in float-float form.
template <class T, class I, bool DFSRC>
__global__ void __launch_bounds__(kPauliTileThreads, 3) pauli_tile_kernel(const PauliTileParams<I> p) {
    using Gm = PtGeom<T>;
    constexpr int E = Gm::E, NA = Gm::NA, NP = Gm::NP, EB = 1 << Gm::LEB;
    constexpr int W = kPauliTileThreads / 32;
    extern __shared__ __align__(128) unsigned char pt_smem[];
    double *slot = reinterpret_cast<double *>(pt_smem + 2 * E * EB);  // [nw][W], after the two tile buffers
    const int tid = threadIdx.x;
    for (int i = tid; i < p.nw * W; i += kPauliTileThreads) slot[i] = 0.0;
    const int lane = tid & 31, warp = tid >> 5;
    const uint32_t lowmask = (1u << p.m) - 1u;
    // 16-byte chunks: two complex64 or one complex128 amplitude each
    constexpr int EPC = sizeof(T) == 4 ? 2 : 1;
    constexpr int GEB = sizeof(T) == 4 ? 8 : 16;  // bytes per amplitude in the state
    const unsigned char *src = static_cast<const unsigned char *>(p.sv);
    auto load = [&](I tau, unsigned char *dst) {
        const I base = insert_holes<I>(tau, p.holes);
        for (int c = tid; c < E / EPC; c += kPauliTileThreads) {
            const uint32_t e = uint32_t(c * EPC);
            const I gi = base + p.hi_off[e >> p.m] + I(e & lowmask);
            pt_cp_async16(dst + size_t(e) * EB, src + size_t(gi) * GEB);
        }
        asm volatile("cp.async.commit_group;" ::: "memory");
    };
    TileAcc<T> acc[kTileWords];  // per-thread sums over all tiles of this CTA
    const I G = I(gridDim.x);
    I tau = blockIdx.x;
    if (tau < p.ntiles) load(tau, pt_smem);
    else asm volatile("cp.async.commit_group;" ::: "memory");
    __syncthreads();
    for (int it = 0; tau < p.ntiles; tau += G, it++) {
        unsigned char *cur = pt_smem + (it & 1) * (E * EB);
        if (tau + G < p.ntiles) load(tau + G, pt_smem + ((it + 1) & 1) * (E * EB));
        else asm volatile("cp.async.commit_group;" ::: "memory");
        asm volatile("cp.async.wait_group 1;" ::: "memory");
        __syncthreads();
        if constexpr (sizeof(T) == 8 && !DFSRC) {  // complex128 -> float-float in place
#pragma unroll 4
            for (int j = 0; j < NA; j++) {
                const int e = tid + j * kPauliTileThreads;
                const double2 v = reinterpret_cast<const double2 *>(cur)[e];
                const DF r = df_from_double(v.x), im = df_from_double(v.y);
                reinterpret_cast<float4 *>(cur)[e] = make_float4(r.hi, im.hi, r.lo, im.lo);
            }
            __syncthreads();
        }
        const I base = insert_holes<I>(tau, p.holes);
        // diagonal words: |a_e|^2 once per element
        if (p.nd > 0) {
            uint32_t pd[kTileWords];
#pragma unroll
            for (int t = 0; t < kTileWords; t++)
                pd[t] = uint32_t(__popc(uint32_t(tid) & p.tsign[t]) + __popcll(uint64_t(base) & p.osign[t])) << 31;
            if constexpr (sizeof(T) == 4) {
#pragma unroll
                for (int j = 0; j < NA; j++) {
                    const float2 a = reinterpret_cast<const float2 *>(cur)[tid + j * kPauliTileThreads];
                    const float q = fmaf(a.x, a.x, a.y * a.y);
#pragma unroll
                    for (int t = 0; t < kTileWords; t++) {
                        if (t >= p.nd) break;
                        acc[t].v += pt_flip_sign(q, pd[t] ^ p.cs[t][j]);
                    }
                }
            } else {
                // elements j and j + 1 in the two lanes
#pragma unroll
                for (int j = 0; j < NA; j += 2) {
                    float qh[2], ql[2];
#pragma unroll
                    for (int u = 0; u < 2; u++) {
                        const float4 a =
                            reinterpret_cast<const float4 *>(cur)[tid + (j + u) * kPauliTileThreads];  // (rh, ih, rl, il)
                        const float p1 = df_mul_rn(a.x, a.x), p2 = df_mul_rn(a.y, a.y);
                        float l = df_add_rn(df_fma(a.x, a.x, -p1), df_fma(a.y, a.y, -p2));
                        l = df_fma(df_add_rn(a.x, a.x), a.z, l);
                        l = df_fma(df_add_rn(a.y, a.y), a.w, l);
                        const float h = df_add_rn(p1, p2);
                        const float bb = df_sub_rn(h, p1);
                        ql[u] = df_add_rn(l, df_add_rn(df_sub_rn(p1, df_sub_rn(h, bb)), df_sub_rn(p2, bb)));
                        qh[u] = h;
                    }
                    const F2 qh2 = f2_pack(qh[0], qh[1]), ql2 = f2_pack(ql[0], ql[1]);
#pragma unroll
                    for (int t = 0; t < kTileWords; t++) {
                        if (t >= p.nd) break;
                        df2_acc_signed(acc[t].v, pd[t] ^ p.cs[t][j], pd[t] ^ p.cs[t][j + 1], qh2, ql2);
                    }
                }
            }
        }
        // words with flips
#pragma unroll
        for (int t = 0; t < kTileWords; t++) {
            if (t >= p.nw) break;
            if (t < p.nd) continue;
            const uint32_t X = pt_insert_zero(uint32_t(tid), p.b0[t]);
            const uint32_t P =
                uint32_t(__popc(X & p.tsign[t]) + __popcll(uint64_t(base) & p.osign[t])) << 31;
            const unsigned char *pa = cur + (X << Gm::LEB);
            const unsigned char *pb = cur + ((X << Gm::LEB) ^ p.fxb[t]);
            const bool im = (p.use_im >> t) & 1u;
            if constexpr (sizeof(T) == 4) {
                if (im) {
#pragma unroll
                    for (int j = 0; j < NP; j++) {
                        const float2 a = *reinterpret_cast<const float2 *>(pa + p.ja[t][j]);
                        const float2 b = *reinterpret_cast<const float2 *>(pb + p.jb[t][j]);
                        acc[t].v += pt_flip_sign(fmaf(a.x, b.y, -a.y * b.x), P ^ p.cs[t][j]);
                    }
                } else {
#pragma unroll
                    for (int j = 0; j < NP; j++) {
                        const float2 a = *reinterpret_cast<const float2 *>(pa + p.ja[t][j]);
                        const float2 b = *reinterpret_cast<const float2 *>(pb + p.jb[t][j]);
                        acc[t].v += pt_flip_sign(fmaf(a.x, b.x, a.y * b.y), P ^ p.cs[t][j]);
                    }
                }
            } else {
                // lanes: the two products of Re or Im of conj(a) b
                if (im) {  // (ar bi, -ai br)
#pragma unroll
                    for (int j = 0; j < NP; j++) {
                        const float4 a = *reinterpret_cast<const float4 *>(pa + p.ja[t][j]);
                        const float4 b = *reinterpret_cast<const float4 *>(pb + p.jb[t][j]);
                        const uint32_t sb = P ^ p.cs[t][j];
                        df2_acc_mul(acc[t].v, sb, sb ^ 0x80000000u, DF2{f2_pack(a.x, a.y), f2_pack(a.z, a.w)},
                                    DF2{f2_pack(b.y, b.x), f2_pack(b.w, b.z)});
                    }
                } else {  // (ar br, ai bi)
#pragma unroll
                    for (int j = 0; j < NP; j++) {
                        const float4 a = *reinterpret_cast<const float4 *>(pa + p.ja[t][j]);
                        const float4 b = *reinterpret_cast<const float4 *>(pb + p.jb[t][j]);
                        const uint32_t sb = P ^ p.cs[t][j];
                        df2_acc_mul(acc[t].v, sb, sb, DF2{f2_pack(a.x, a.y), f2_pack(a.z, a.w)},
                                    DF2{f2_pack(b.x, b.y), f2_pack(b.z, b.w)});
                    }
                }
            }
        }
        __syncthreads();  // `cur` is the target of a load issued next iteration
    }
    asm volatile("cp.async.wait_group 0;" ::: "memory");
#pragma unroll
    for (int t = 0; t < kTileWords; t++) {
        if (t >= p.nw) break;
        acc[t].warp_reduce();
        if (lane == 0) slot[t * W + warp] = acc[t].value();
    }
    __syncthreads();
    for (int t = tid; t < p.nw; t += kPauliTileThreads) {
        double v = 0.0;
        for (int w = 0; w < W; w++) v += slot[t * W + w];
        p.partials[size_t(blockIdx.x) * p.nw + t] = v;
    }
}

// out[t] = the sum over CTAs of the partials: one warp per word, lane l sums
// the CTAs l, l + 32, ... in order, then a fixed shuffle tree adds the lanes.
__global__ void pauli_tile_reduce(const double *__restrict__ partials, int nctas, int nw, double *__restrict__ out) {
    const int t = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (t >= nw) return;  // whole warps leave together
    double v = 0.0;
    for (int c = lane; c < nctas; c += 32) v += partials[size_t(c) * nw + t];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) out[t] = v;
}

// Raw sums of the words (as the Walsh-Hadamard pass defines them) by tile
// passes; done[w] = 0 for the words whose flip mask fits no tile.
template <class T, class I>
static lgpu_status_t pauli_tile_raw(lgpu_context_t ctx, const void *sv, uint32_t n, uint32_t nwords,
                                    const uint64_t *flip, const uint64_t *sign, std::vector<double> &raw,
                                    std::vector<char> &done, cudaStream_t s) {
    using Gm = PtGeom<T>;
    done.assign(nwords, 0);
    raw.assign(nwords, 0.0);
    if (n < uint32_t(Gm::K)) return LGPU_OK;
    const auto passes = plan_tile_passes(n, nwords, flip, Gm::K, Gm::MMIN);
    if (passes.empty()) return LGPU_OK;
    const unsigned sms = unsigned(sm_count());
    const unsigned grid_cap = sms * 3;
    void *scr = nullptr;
    const size_t pbytes = sizeof(double) * size_t(grid_cap) * kTileWords;
    const size_t rbytes = sizeof(double) * passes.size() * kTileWords;
    LGPU_TRY(ctx_scratch(ctx, 256 + pbytes + rbytes, &scr));
    double *partials = reinterpret_cast<double *>(static_cast<char *>(scr) + 256);
    double *results = reinterpret_cast<double *>(static_cast<char *>(scr) + 256 + pbytes);
    static std::atomic<size_t> attr[64], attr_df[64];
    // complex128 over three or more passes: convert the state to float-float
    // once (one read and one write of the state) instead of in every pass,
    // when a copy of the state's size takes at most a quarter of the free memory
    void *dfcopy = nullptr;
    const size_t svbytes = (size_t(1) << n) * sizeof(cplx_t<T>);
    if (sizeof(T) == 8 && passes.size() >= 3) {
        size_t freeb = 0, totalb = 0;
        if (cudaMemGetInfo(&freeb, &totalb) == cudaSuccess && svbytes <= freeb / 4) {
            if (cudaMallocAsync(&dfcopy, svbytes, s) != cudaSuccess) {
                cudaGetLastError();
                dfcopy = nullptr;
            }
        } else {
            cudaGetLastError();
        }
    }
    struct FreeOnExit {
        void *p;
        cudaStream_t s;
        ~FreeOnExit() {
            if (p) cudaFreeAsync(p, s);
        }
    } df_guard{dfcopy, s};
    if (dfcopy) {
        const uint64_t count = uint64_t(1) << n;
        const unsigned g = grid_for(count, 256, 8, 8);
        df_state_copy_kernel<<<g, 256, 0, s>>>(static_cast<const double2 *>(sv), static_cast<float4 *>(dfcopy), count);
        LGPU_CHECK_LAUNCH();
    }
    std::vector<std::vector<uint32_t>> order(passes.size());  // word of each result slot
    for (size_t pi = 0; pi < passes.size(); pi++) {
        const TilePass &tp = passes[pi];
        const int k = int(tp.tile.size());
        if (k != Gm::K) return fail(LGPU_ERR_UNSUPPORTED, "Pauli tile pass of unexpected size");
        int m = 0;
        while (m < k && tp.tile[size_t(m)] == m) m++;
        auto b = std::make_unique<PauliTileParams<I>>();
        std::memset(b.get(), 0, sizeof(PauliTileParams<I>));
        b->sv = sv;
        b->holes = make_holes(tp.tile);
        b->ntiles = I(uint64_t(1) << (n - uint32_t(k)));
        b->m = m;
        for (int h = 0; h < (1 << (k - m)); h++) {
            uint64_t o = 0;
            for (int q = m; q < k; q++)
                if ((h >> (q - m)) & 1) o |= uint64_t(1) << tp.tile[size_t(q)];
            b->hi_off[h] = I(o);
        }
        // diagonal words first
        auto &ord = order[pi];
        for (uint32_t w : tp.words)
            if (flip[w] == 0) ord.push_back(w);
        b->nd = int(ord.size());
        for (uint32_t w : tp.words)
            if (flip[w] != 0) ord.push_back(w);
        b->nw = int(ord.size());
        for (int t = 0; t < b->nw; t++) {
            const uint32_t w = ord[size_t(t)];
            uint32_t tf = 0, ts = 0;
            uint64_t os = sign[w];
            for (int q = 0; q < k; q++) {
                const int bit = tp.tile[size_t(q)];
                if ((flip[w] >> bit) & 1u) tf |= 1u << q;
                if ((sign[w] >> bit) & 1u) {
                    ts |= 1u << q;
                    os &= ~(uint64_t(1) << bit);
                }
            }
            b->tsign[t] = ts;
            b->osign[t] = os;
            if (flip[w] && (__builtin_popcountll(flip[w] & sign[w]) & 1)) b->use_im |= 1u << t;
            if (tf == 0) {
                for (int j = 0; j < Gm::NA; j++)
                    b->cs[t][j] = uint32_t(__builtin_popcount((uint32_t(j) << 8) & ts) & 1) << 31;
                continue;
            }
            const uint32_t b0 = uint32_t(__builtin_ctz(tf));
            auto ins = [&](uint32_t v) { return ((v & ~((1u << b0) - 1u)) << 1) | (v & ((1u << b0) - 1u)); };
            const uint32_t jm = ins(uint32_t(Gm::NP - 1) << 8);
            b->b0[t] = b0;
            b->fxb[t] = (tf & ~jm) << Gm::LEB;
            for (int j = 0; j < Gm::NP; j++) {
                const uint32_t J = ins(uint32_t(j) << 8);
                b->ja[t][j] = J << Gm::LEB;
                b->jb[t][j] = (J ^ (tf & jm)) << Gm::LEB;
                b->cs[t][j] = uint32_t(__builtin_popcount(J & ts) & 1) << 31;
            }
        }
        const size_t smem = 2 * size_t(Gm::E) * (size_t(1) << Gm::LEB) + sizeof(double) * size_t(b->nw) * 8;
        const unsigned grid = unsigned(std::min<uint64_t>(uint64_t(b->ntiles), grid_cap));
        b->partials = partials;
        bool launched = false;
        if constexpr (sizeof(T) == 8) {
            if (dfcopy) {
                b->sv = dfcopy;
                LGPU_TRY(ensure_smem(reinterpret_cast<const void *>(pauli_tile_kernel<T, I, true>), smem, attr_df));
                pauli_tile_kernel<T, I, true><<<grid, kPauliTileThreads, smem, s>>>(*b);
                launched = true;
            }
        }
        if (!launched) {
            LGPU_TRY(ensure_smem(reinterpret_cast<const void *>(pauli_tile_kernel<T, I, false>), smem, attr));
            pauli_tile_kernel<T, I, false><<<grid, kPauliTileThreads, smem, s>>>(*b);
        }
        LGPU_CHECK_LAUNCH();
        pauli_tile_reduce<<<1, 32 * kTileWords, 0, s>>>(partials, int(grid), b->nw, results + pi * kTileWords);
        LGPU_CHECK_LAUNCH();
    }
    std::vector<double> host(passes.size() * kTileWords);
    void *pin = nullptr;
    LGPU_TRY(ctx_pinned(ctx, rbytes, &pin));
    LGPU_CUDA_TRY(cudaMemcpyAsync(pin, results, rbytes, cudaMemcpyDeviceToHost, s));
    LGPU_CUDA_TRY(cudaStreamSynchronize(s));
    std::memcpy(host.data(), pin, rbytes);
    for (size_t pi = 0; pi < passes.size(); pi++)
        for (size_t t = 0; t < order[pi].size(); t++) {
            raw[order[pi][t]] = host[pi * kTileWords + t];
            done[order[pi][t]] = 1;
        }
    return LGPU_OK;
}

template <class T, class I>
static lgpu_status_t pauli_words_t(lgpu_context_t ctx, const void *sv, uint32_t n, uint32_t nwords,
                                   const uint64_t *flip, const uint64_t *sign, const uint8_t *ny, double *out,
                                   int out_on_device, cudaStream_t s, bool tiles = true) {
    // Group words by flip mask (stable order of first appearance).
    std::vector<uint64_t> keys;
    std::vector<std::vector<uint32_t>> groups;
    for (uint32_t w = 0; w < nwords; w++) {
        size_t gi = 0;
        for (; gi < keys.size(); gi++)
            if (keys[gi] == flip[w]) break;
        if (gi == keys.size()) {
            keys.push_back(flip[w]);
            groups.emplace_back();
        }
        groups[gi].push_back(w);
    }
    // Large states with several flip masks: tile passes hold words with
    // different flip masks (one read of the state for several masks).
    if (tiles && n >= 16 && keys.size() >= 2) {
        std::vector<double> raw;
        std::vector<char> done;
        LGPU_TRY((pauli_tile_raw<T, I>(ctx, sv, n, nwords, flip, sign, raw, done, s)));
        // words whose flips fit no tile: the flip-mask passes, as a subset
        std::vector<uint32_t> rest;
        for (uint32_t w = 0; w < nwords; w++)
            if (!done[w]) rest.push_back(w);
        {
            std::vector<double> vals(nwords, 0.0);
            if (!rest.empty()) {
                std::vector<uint64_t> rf, rs;
                std::vector<uint8_t> rn;
                for (uint32_t w : rest) {
                    rf.push_back(flip[w]);
                    rs.push_back(sign[w]);
                    rn.push_back(ny[w]);
                }
                std::vector<double> rv(rest.size());
                LGPU_TRY((pauli_words_t<T, I>(ctx, sv, n, uint32_t(rest.size()), rf.data(), rs.data(), rn.data(),
                                              rv.data(), 0, s, false)));
                for (size_t i = 0; i < rest.size(); i++) vals[rest[i]] = rv[i];
            }
            for (uint32_t w = 0; w < nwords; w++) {
                if (!done[w]) continue;
                const bool kneg = (__builtin_popcountll(flip[w] & sign[w]) & 1) != 0;
                const double x = (!flip[w] ? 1.0 : (kneg ? -2.0 : 2.0)) * raw[w];
                const bool im = flip[w] && kneg;
                const double vx = im ? 0.0 : x, vy = im ? x : 0.0;
                switch (ny[w] & 3) {  // <P> = Re(i^ny * (vx + i vy))
                case 0: vals[w] = vx; break;
                case 1: vals[w] = -vy; break;
                case 2: vals[w] = -vx; break;
                default: vals[w] = vy; break;
                }
            }
            if (out_on_device) {
                LGPU_CUDA_TRY(cudaMemcpyAsync(out, vals.data(), nwords * sizeof(double), cudaMemcpyHostToDevice, s));
                LGPU_CUDA_TRY(cudaStreamSynchronize(s));
            } else {
                std::memcpy(out, vals.data(), nwords * sizeof(double));
            }
            return LGPU_OK;
        }
    }
    if (n >= 4) {
        // Walsh-Hadamard passes: up to kWhtWords words sharing one flip mask.
        struct WPass {
            uint64_t flip;
            std::vector<uint32_t> words;
        };
        std::vector<WPass> wp;
        for (size_t gi = 0; gi < keys.size(); gi++)
            for (size_t o = 0; o < groups[gi].size(); o += kWhtWords)
                wp.push_back({keys[gi], std::vector<uint32_t>(groups[gi].begin() + o,
                                                              groups[gi].begin() + std::min(groups[gi].size(),
                                                                                            o + kWhtWords))});
        const uint64_t N = uint64_t(1) << n;
        const unsigned g = reduce_grid(N / 8);
        void *p = nullptr;
        const size_t pbytes = size_t(g) * kWhtWords * sizeof(double2);
        const size_t rbytes = wp.size() * kWhtWords * sizeof(double2);
        LGPU_TRY(ctx_scratch(ctx, 256 + pbytes + rbytes, &p));
        auto *counter = static_cast<unsigned *>(p);
        auto *partials = reinterpret_cast<double2 *>(static_cast<char *>(p) + 256);
        auto *results = reinterpret_cast<double2 *>(static_cast<char *>(p) + 256 + pbytes);
        std::vector<double> coef(wp.size() * kWhtWords, 0.0);
        for (size_t pi = 0; pi < wp.size(); pi++) {
            PauliWhtParams<T, I> b{};
            b.sv = static_cast<const cplx_t<T> *>(sv);
            b.flip = I(wp[pi].flip);
            std::vector<int> hole;
            if (wp[pi].flip) hole.push_back(__builtin_ctzll(wp[pi].flip));
            b.holes = make_holes(hole);
            const uint64_t items = wp[pi].flip ? N / 2 : N;
            b.slots = I(items / 8);
            b.lgS = __builtin_ctzll(items / 8);
            b.nt = int(wp[pi].words.size());
            // element positions of the three j bits
            int pj[3];
            for (int q = 0; q < 3; q++) {
                int pos = b.lgS + q;
                if (!hole.empty() && pos >= hole[0]) pos++;
                pj[q] = pos;
            }
            // one word's coefficient directly costs 7 adds, the full transform 24 per product array
            b.direct = b.nt <= kDirectWords ? 1 : 0;
            for (int t = 0; t < b.nt; t++) {
                const uint32_t w = wp[pi].words[size_t(t)];
                b.sgn[t] = I(sign[w]);
                uint32_t h = 0;
                for (int q = 0; q < 3; q++) h |= uint32_t((sign[w] >> pj[q]) & 1u) << q;
                b.hsel[t] = h;
                const bool kneg = (__builtin_popcountll(flip[w] & sign[w]) & 1) != 0;
                if (wp[pi].flip && kneg) b.use_im |= 1u << t;
                if (wp[pi].flip && kneg) b.need_im = 1;
                else b.need_re = 1;
                // v.x = sum(+-w) (flip 0) or 2 sum(+-Re w); v.y = -2 sum(+-Im w) (odd flip/sign overlap)
                coef[pi * kWhtWords + size_t(t)] = !wp[pi].flip ? 1.0 : (kneg ? -2.0 : 2.0);
            }
            if (b.direct)
                LGPU_TRY((wht_dispatch<T, I, true>(b, g, partials, counter, results + pi * kWhtWords, s)));
            else
                LGPU_TRY((wht_dispatch<T, I, false>(b, g, partials, counter, results + pi * kWhtWords, s)));
        }
        std::vector<double2> host(wp.size() * kWhtWords);
        if (!wp.empty()) {
            void *pin = nullptr;
            LGPU_TRY(ctx_pinned(ctx, rbytes, &pin));
            LGPU_CUDA_TRY(cudaMemcpyAsync(pin, results, rbytes, cudaMemcpyDeviceToHost, s));
            LGPU_CUDA_TRY(cudaStreamSynchronize(s));
            std::memcpy(host.data(), pin, rbytes);
        }
        std::vector<double> vals(nwords, 0.0);
        for (size_t pi = 0; pi < wp.size(); pi++)
            for (size_t t = 0; t < wp[pi].words.size(); t++) {
                const uint32_t w = wp[pi].words[t];
                const double x = coef[pi * kWhtWords + t] * host[pi * kWhtWords + t].x;
                const bool im = wp[pi].flip && (__builtin_popcountll(flip[w] & sign[w]) & 1);
                const double vx = im ? 0.0 : x, vy = im ? x : 0.0;
                // <P> = Re(i^ny * (vx + i vy))
                double re = 0;
                switch (ny[w] & 3) {
                case 0: re = vx; break;
                case 1: re = -vy; break;
                case 2: re = -vx; break;
                default: re = vy; break;
                }
                vals[w] = re;
            }
        if (out_on_device) {
            LGPU_CUDA_TRY(cudaMemcpyAsync(out, vals.data(), nwords * sizeof(double), cudaMemcpyHostToDevice, s));
            LGPU_CUDA_TRY(cudaStreamSynchronize(s));
        } else {
            std::memcpy(out, vals.data(), nwords * sizeof(double));
        }
        return LGPU_OK;
    }
    // Small states: up to kWordsPerPass words sharing one flip mask per pass.
    struct Pass {
        uint64_t flip;
        std::vector<uint32_t> words;
    };
    std::vector<Pass> passes;
    for (size_t gi = 0; gi < keys.size(); gi++)
        for (size_t o = 0; o < groups[gi].size(); o += kWordsPerPass)
            passes.push_back({keys[gi], std::vector<uint32_t>(groups[gi].begin() + o,
                                                               groups[gi].begin() + std::min(groups[gi].size(),
                                                                                             o + kWordsPerPass))});
    const uint64_t N = uint64_t(1) << n;
    const unsigned g = reduce_grid(N);
    // scratch: counter | partials (g * 8) | results (passes * 8)
    void *p = nullptr;
    const size_t pbytes = size_t(g) * kWordsPerPass * sizeof(double2);
    const size_t rbytes = passes.size() * kWordsPerPass * sizeof(double2);
    LGPU_TRY(ctx_scratch(ctx, 256 + pbytes + rbytes, &p));
    auto *counter = static_cast<unsigned *>(p);
    auto *partials = reinterpret_cast<double2 *>(static_cast<char *>(p) + 256);
    auto *results = reinterpret_cast<double2 *>(static_cast<char *>(p) + 256 + pbytes);
    for (size_t pi = 0; pi < passes.size(); pi++) {
        PauliBody<T, I> b{};
        b.sv = static_cast<const cplx_t<T> *>(sv);
        b.flip = I(passes[pi].flip);
        std::vector<int> hole;
        if (passes[pi].flip) hole.push_back(__builtin_ctzll(passes[pi].flip));
        b.holes = make_holes(hole);
        b.nt = int(passes[pi].words.size());
        for (int t = 0; t < b.nt; t++) {
            const uint32_t w = passes[pi].words[size_t(t)];
            b.sgn[t] = I(sign[w]);
            b.kappa_neg[t] = __builtin_popcountll(flip[w] & sign[w]) & 1;
        }
        const uint64_t items = passes[pi].flip ? N / 2 : N;
        reduce_kernel<kWordsPerPass, I><<<g, kReduceBlock, 0, s>>>(b, I(items), partials, counter,
                                                                   results + pi * kWordsPerPass);
        LGPU_CHECK_LAUNCH();
    }
    std::vector<double2> host(passes.size() * kWordsPerPass);
    if (!passes.empty()) {
        void *pin = nullptr;
        LGPU_TRY(ctx_pinned(ctx, rbytes, &pin));
        LGPU_CUDA_TRY(cudaMemcpyAsync(pin, results, rbytes, cudaMemcpyDeviceToHost, s));
        LGPU_CUDA_TRY(cudaStreamSynchronize(s));
        std::memcpy(host.data(), pin, rbytes);
    }
    std::vector<double> vals(nwords, 0.0);
    for (size_t pi = 0; pi < passes.size(); pi++)
        for (size_t t = 0; t < passes[pi].words.size(); t++) {
            const uint32_t w = passes[pi].words[t];
            const double2 v = host[pi * kWordsPerPass + t];
            // <P> = Re(i^ny * (v.x + i v.y))
            double re = 0;
            switch (ny[w] & 3) {
            case 0: re = v.x; break;
            case 1: re = -v.y; break;
            case 2: re = -v.x; break;
            default: re = v.y; break;
            }
            vals[w] = re;
        }
    if (out_on_device)
        LGPU_CUDA_TRY(cudaMemcpyAsync(out, vals.data(), nwords * sizeof(double), cudaMemcpyHostToDevice, s));
    else
        std::memcpy(out, vals.data(), nwords * sizeof(double));
    if (out_on_device) LGPU_CUDA_TRY(cudaStreamSynchronize(s));
    return LGPU_OK;
}

// ---------------------------------------------------------------------------
// |a|^2 without FP64 instructions (GB300 issues about 2 FP64 operations per
// clock per SM, so one DFMA + DMUL + DADD per amplitude would bound these
// single-read passes at a third of HBM bandwidth): the square is formed in
// float-float (exact for complex64; complex128 is split to float-float
// first), short runs are summed in float-float and each run's sum is added
// to a double.
// ---------------------------------------------------------------------------
__device__ __forceinline__ DF prob_df(const float2 a) {
    const float px = df_mul_rn(a.x, a.x), py = df_mul_rn(a.y, a.y);
    return df_sum<2>({DF{px, df_fma(a.x, a.x, -px)}, DF{py, df_fma(a.y, a.y, -py)}});
}
__device__ __forceinline__ DF prob_df(const double2 a) {
    const DF x = df_from_double(a.x), y = df_from_double(a.y);
    return df_sum<2>({df_mul(x, x), df_mul(y, y)});
}

// Sum of |a_i|^2 over i = start + STRIDE j < len (one thread's share of a
// slice): eight loads in flight per thread.
template <class T, class I, int STRIDE>
__device__ __forceinline__ double strided_prob_sum(const cplx_t<T> *__restrict__ a, I len, int start) {
    double acc = 0.0;
    for (I o = I(start); o < len; o += I(STRIDE * 8)) {
        cplx_t<T> v[8];
#pragma unroll
        for (int u = 0; u < 8; u++) {
            const I i = o + I(STRIDE * u);
            v[u] = i < len ? a[i] : cplx_t<T>{};
        }
        DF run = prob_df(v[0]);
#pragma unroll
        for (int u = 1; u < 8; u++) run = df_sum<2>({run, prob_df(v[u])});
        acc += df_to_double(run);
    }
    return acc;
}

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// ---------------------------------------------------------------------------
// Probabilities
// ---------------------------------------------------------------------------
struct BinMap {
    int k;
    int bits[24];
};

template <class I> __device__ __forceinline__ uint32_t bin_of(I i, const BinMap &bm) {
    uint32_t b = 0;
#pragma unroll 4
    for (int q = 0; q < bm.k; q++) b |= uint32_t((i >> bm.bits[q]) & 1) << q;
    return b;
}

// Marginal histogram over chunks of 2^chunk_log2 amplitudes.  Bins are split
// into the probed bits at or above chunk_log2 (constant over a chunk) and
// those below it.  Without low bits a chunk feeds one bin: each warp sums a
// slice and adds it to the CTA's histogram once.  With low bits every thread
// accumulates runs of equal bin over its strided amplitudes.
template <class T, class I>
__global__ void __launch_bounds__(256)
    probs_hist_kernel(const cplx_t<T> *__restrict__ sv, I N, int chunk_log2, BinMap bm, double *partials,
                      unsigned *counter, double *out) {
    extern __shared__ double hist[];
    const int nb = 1 << bm.k;
    for (int b = threadIdx.x; b < nb; b += 256) hist[b] = 0.0;
    uint32_t lowsel = 0;  // probed bits below chunk_log2 (output bit positions)
    for (int q = 0; q < bm.k; q++)
        if (bm.bits[q] < chunk_log2) lowsel |= 1u << q;
    __syncthreads();
    const I chunk = I(1) << chunk_log2;
    const I nchunks = N >> chunk_log2;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (I c = blockIdx.x; c < nchunks; c += gridDim.x) {
        const I base = c * chunk;
        uint32_t hb = 0;
        for (int q = 0; q < bm.k; q++)
            if (!((lowsel >> q) & 1u)) hb |= uint32_t((base >> bm.bits[q]) & 1) << q;
        if (lowsel == 0 && chunk_log2 >= 8) {
            const I per = chunk >> 3;  // eight warps, one slice each (>= 32 amplitudes)
            const double v = warp_sum_d(strided_prob_sum<T, I, 32>(sv + base + I(warp) * per, per, lane));
            if (lane == 0) atomicAdd(&hist[hb], v);
            continue;
        }
        // A thread visits offsets threadIdx.x + 256 j: probed bits below 8
        // are fixed for it, so without probed bits in [8, chunk_log2) its
        // whole share of the chunk feeds one bin.
        uint32_t tb = hb, midsel = 0;
        for (int q = 0; q < bm.k; q++)
            if ((lowsel >> q) & 1u) {
                if (bm.bits[q] < 8) tb |= uint32_t((threadIdx.x >> bm.bits[q]) & 1) << q;
                else midsel |= 1u << q;
            }
        if (midsel == 0) {
            if (I(threadIdx.x) < chunk) atomicAdd(&hist[tb], strided_prob_sum<T, I, 256>(sv + base, chunk, threadIdx.x));
            continue;
        }
        uint32_t cur = 0xffffffffu;
        DF run{0.0f, 0.0f};
        for (I o = threadIdx.x; o < chunk; o += 256) {
            const DF pr = prob_df(sv[base + o]);
            uint32_t b = hb;
            for (int q = 0; q < bm.k; q++)
                if ((lowsel >> q) & 1u) b |= uint32_t((o >> bm.bits[q]) & 1) << q;
            if (b != cur) {
                if (cur != 0xffffffffu) atomicAdd(&hist[cur], df_to_double(run));
                cur = b;
                run = pr;
            } else {
                run = df_sum<2>({run, pr});
            }
        }
        if (cur != 0xffffffffu) atomicAdd(&hist[cur], df_to_double(run));
    }
    __syncthreads();
    for (int b = threadIdx.x; b < nb; b += 256) partials[size_t(blockIdx.x) * nb + b] = hist[b];
    if (last_block_arrive(counter)) {
        for (int b = threadIdx.x; b < nb; b += 256) {
            double s = 0.0;
            for (unsigned k = 0; k < gridDim.x; k++) s += __ldcg(&partials[size_t(k) * nb + b]);
            out[b] = s;
        }
        if (threadIdx.x == 0) *counter = 0u;
    }
}

template <class T, class I>
__global__ void probs_atomic_kernel(const cplx_t<T> *__restrict__ sv, I N, BinMap bm, double *out) {
    const I stride = I(gridDim.x) * blockDim.x;
    for (I i = I(blockIdx.x) * blockDim.x + threadIdx.x; i < N; i += stride) {
        atomicAdd(&out[bin_of<I>(i, bm)], df_to_double(prob_df(sv[i])));
    }
}

// Marginal probabilities when every probed bit is at or above chunk_log2:
// each chunk feeds one bin.  One CTA per bin sums the chunk sums csum[c] of
// that bin in a fixed order.  The chunk index has m = n - chunk_log2 bits;
// the probed ones are fixed by the bin, the others enumerate the bin's chunks.
__global__ void __launch_bounds__(256)
    probs_from_chunks_kernel(const double *__restrict__ csum, int m, int chunk_log2, BinMap bm, double *out) {
    __shared__ double2 sm[8];
    const uint32_t b = blockIdx.x;
    uint64_t fixed = 0, probed = 0;
    for (int q = 0; q < bm.k; q++) {
        const int cb = bm.bits[q] - chunk_log2;
        probed |= uint64_t(1) << cb;
        if ((b >> q) & 1u) fixed |= uint64_t(1) << cb;
    }
    const uint64_t freemask = ((uint64_t(1) << m) - 1) & ~probed;
    const uint64_t per_bin = uint64_t(1) << (m - bm.k);
    double acc = 0.0;
    for (uint64_t j = threadIdx.x; j < per_bin; j += 256) {
        uint64_t c = fixed, jj = j;
        for (uint64_t fm = freemask; fm && jj; fm &= fm - 1, jj >>= 1)
            if (jj & 1) c |= fm & (0 - fm);
        acc += csum[c];
    }
    const double2 v = block_reduce_d2<256>(make_double2(acc, 0.0), sm);
    if (threadIdx.x == 0) out[b] = v.x;
}

template <class T>
__global__ void __launch_bounds__(256)
    chunk_sums_kernel(const cplx_t<T> *__restrict__ sv, uint64_t nchunks, int chunk_log2, double *csum);

template <class T, class I>
static lgpu_status_t probs_t(lgpu_context_t ctx, const void *svv, uint32_t n, const std::vector<int> &bits,
                             double *out, int out_on_device, cudaStream_t s) {
    const auto *sv = static_cast<const cplx_t<T> *>(svv);
    BinMap bm{};
    bm.k = int(bits.size());
    for (int q = 0; q < bm.k; q++) bm.bits[q] = bits[size_t(q)];
    const uint64_t N = uint64_t(1) << n;
    const size_t nb = size_t(1) << bm.k;
    void *p = nullptr;
    double *res = nullptr;
    int minbit = int(n);
    for (int b : bits) minbit = std::min(minbit, b);
    // chunks of >= 1024 amplitudes, at most 2^20 of them, each inside one bin
    const int cl_fast = std::min(minbit, std::max(10, int(n) - 14));
    if (bm.k >= 1 && bm.k <= 12 && cl_fast >= 10 && int(n) - cl_fast <= 20) {
        const uint64_t nchunks = N >> cl_fast;
        LGPU_TRY(ctx_scratch(ctx, 256 + nchunks * sizeof(double) + nb * sizeof(double), &p));
        auto *csum = reinterpret_cast<double *>(static_cast<char *>(p) + 256);
        res = csum + nchunks;
        const unsigned g1 =
            unsigned(std::max<uint64_t>(1, std::min<uint64_t>((nchunks + 7) / 8, uint64_t(sm_count()) * 8)));
        chunk_sums_kernel<T><<<g1, 256, 0, s>>>(sv, nchunks, cl_fast, csum);
        LGPU_CHECK_LAUNCH();
        probs_from_chunks_kernel<<<unsigned(nb), 256, 0, s>>>(csum, int(n) - cl_fast, cl_fast, bm, res);
        LGPU_CHECK_LAUNCH();
    } else if (bm.k <= 12) {
        int chunk_log2 = std::max(8, int(n) - 12);
        if (chunk_log2 > int(n)) chunk_log2 = int(n);
        const uint64_t nchunks = N >> chunk_log2;
        // eight loads in flight per thread; with many bins, two CTAs per SM
        // keep the last CTA's sum over the per-CTA histograms short
        const uint64_t per_sm = nb <= 64 ? 8 : 2;
        const unsigned g = unsigned(std::min<uint64_t>(nchunks, uint64_t(sm_count()) * per_sm));
        LGPU_TRY(ctx_scratch(ctx, 256 + size_t(g) * nb * sizeof(double) + nb * sizeof(double), &p));
        auto *counter = static_cast<unsigned *>(p);
        auto *partials = reinterpret_cast<double *>(static_cast<char *>(p) + 256);
        res = partials + size_t(g) * nb;
        const size_t smem = nb * sizeof(double);
        static std::atomic<size_t> attr_p[64];
        LGPU_TRY(ensure_smem(reinterpret_cast<const void *>(probs_hist_kernel<T, I>), smem, attr_p));
        if (n < 8) chunk_log2 = int(n);
        probs_hist_kernel<T, I><<<g, 256, smem, s>>>(sv, I(N), chunk_log2, bm, partials, counter, res);
        LGPU_CHECK_LAUNCH();
    } else {
        LGPU_TRY(ctx_scratch(ctx, 256 + nb * sizeof(double), &p));
        res = reinterpret_cast<double *>(static_cast<char *>(p) + 256);
        LGPU_CUDA_TRY(cudaMemsetAsync(res, 0, nb * sizeof(double), s));
        probs_atomic_kernel<T, I><<<grid_for(N, 256, 4), 256, 0, s>>>(sv, I(N), bm, res);
        LGPU_CHECK_LAUNCH();
    }
    if (out_on_device) {
        LGPU_CUDA_TRY(cudaMemcpyAsync(out, res, nb * sizeof(double), cudaMemcpyDeviceToDevice, s));
        return LGPU_OK;
    }
    LGPU_CUDA_TRY(cudaMemcpyAsync(out, res, nb * sizeof(double), cudaMemcpyDeviceToHost, s));
    LGPU_CUDA_TRY(cudaStreamSynchronize(s));
    return LGPU_OK;
}

// ---------------------------------------------------------------------------
// Sampling
// ---------------------------------------------------------------------------
// csum[c] = sum of |a_i|^2 over chunk c: one warp per chunk.
template <class T>
__global__ void __launch_bounds__(256)
    chunk_sums_kernel(const cplx_t<T> *__restrict__ sv, uint64_t nchunks, int chunk_log2, double *csum) {
    const int lane = threadIdx.x & 31;
    const uint64_t warp = (uint64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const uint64_t nwarps = (uint64_t(gridDim.x) * blockDim.x) >> 5;
    const uint64_t chunk = uint64_t(1) << chunk_log2;
    for (uint64_t c = warp; c < nchunks; c += nwarps) {
        const double v = warp_sum_d(strided_prob_sum<T, uint64_t, 32>(sv + c * chunk, chunk, lane));
        if (lane == 0) csum[c] = v;
    }
}

// Exclusive scan of csum within blocks of 1024 chunks (one CTA each, in
// place); each block's total goes to btot[block].
__global__ void __launch_bounds__(1024) scan_blocks_kernel(double *csum, uint64_t nchunks, double *btot) {
    __shared__ double wsum[32];
    const uint64_t i = uint64_t(blockIdx.x) * 1024 + threadIdx.x;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const double v = i < nchunks ? csum[i] : 0.0;
    double x = v;  // inclusive warp scan
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const double y = __shfl_up_sync(0xffffffffu, x, d);
        if (lane >= d) x += y;
    }
    if (lane == 31) wsum[w] = x;
    __syncthreads();
    if (w == 0) {
        const double t = wsum[lane];
        double z = t;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const double y = __shfl_up_sync(0xffffffffu, z, d);
            if (lane >= d) z += y;
        }
        wsum[lane] = z - t;
        if (lane == 31) btot[blockIdx.x] = z;
    }
    __syncthreads();
    if (i < nchunks) csum[i] = wsum[w] + (x - v);
}

// Exclusive scan of the (at most 256) block totals by one thread; the sum
// of all probabilities goes to *total.
__global__ void scan_tops_kernel(double *btot, uint32_t nblocks, double *total) {
    if (threadIdx.x != 0) return;
    double run = 0.0;
    for (uint32_t b = 0; b < nblocks; b++) {
        const double v = btot[b];
        btot[b] = run;
        run += v;
    }
    *total = run;
}

// Cumulative probability before chunk c.
__device__ __forceinline__ double chunk_start(const double *csum, const double *boff, uint64_t c) {
    return boff[c >> 10] + csum[c];
}

// One warp per draw.
template <class T>
__global__ void __launch_bounds__(256)
    search_kernel(const cplx_t<T> *__restrict__ sv, const double *__restrict__ cstart,
                  const double *__restrict__ boff, uint64_t nchunks, int chunk_log2, const double *total_p,
                  const double *draws, uint64_t shots, uint64_t *out) {
    const int lane = threadIdx.x & 31;
    const uint64_t warp = (uint64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const uint64_t nwarps = (uint64_t(gridDim.x) * blockDim.x) >> 5;
    const double total = *total_p;
    const uint64_t chunk = uint64_t(1) << chunk_log2;
    for (uint64_t sidx = warp; sidx < shots; sidx += nwarps) {
        const double target = draws[sidx] * total;
        // chunk: last c whose start is <= target (binary search)
        uint64_t lo = 0, hi = nchunks;  // invariant: answer in [lo, hi)
        while (hi - lo > 1) {
            const uint64_t mid = (lo + hi) >> 1;
            if (chunk_start(cstart, boff, mid) <= target)
                lo = mid;
            else
                hi = mid;
        }
        // Walk forward through chunks (handles rounding at chunk borders: a
        // crossing that falls exactly on a border lands on the first index of
        // non-zero probability of a later chunk).
        uint64_t found = ~uint64_t(0), last_nz = ~uint64_t(0);
        for (uint64_t c = lo; c < nchunks && found == ~uint64_t(0); c++) {
            double run = chunk_start(cstart, boff, c);
            for (uint64_t o = 0; o < chunk; o += 32) {
                double p = 0.0;
                if (o + lane < chunk) {
                    const cplx_t<T> a = sv[c * chunk + o + lane];
                    p = fma(double(a.x), double(a.x), double(a.y) * double(a.y));
                }
                double x = p;  // inclusive warp scan
#pragma unroll
                for (int d = 1; d < 32; d <<= 1) {
                    const double y = __shfl_up_sync(0xffffffffu, x, d);
                    if (lane >= d) x += y;
                }
                const double incl = run + x;
                const unsigned hit = __ballot_sync(0xffffffffu, incl > target && p > 0.0);
                const unsigned nz = __ballot_sync(0xffffffffu, p > 0.0);
                if (nz) last_nz = c * chunk + o + (31 - __clz(nz));
                if (hit) {
                    found = c * chunk + o + (__ffs(hit) - 1);
                    break;
                }
                run += __shfl_sync(0xffffffffu, x, 31);
            }
        }
        if (found == ~uint64_t(0)) {
            // Past the end (rounding): the last index of non-zero probability,
            // searched backwards from chunk lo when the walk saw none.
            for (uint64_t c = lo + 1; c-- > 0 && last_nz == ~uint64_t(0);) {
                for (uint64_t o = 0; o < chunk; o += 32) {
                    double p = 0.0;
                    if (o + lane < chunk) {
                        const cplx_t<T> a = sv[c * chunk + o + lane];
                        p = fma(double(a.x), double(a.x), double(a.y) * double(a.y));
                    }
                    const unsigned nz = __ballot_sync(0xffffffffu, p > 0.0);
                    if (nz) last_nz = c * chunk + o + (31 - __clz(nz));
                }
            }
            found = last_nz == ~uint64_t(0) ? 0 : last_nz;
        }
        if (lane == 0) out[sidx] = found;
    }
}

template <class T>
static lgpu_status_t sample_t(lgpu_context_t ctx, const void *svv, uint32_t n, const double *draws, uint64_t shots,
                              uint64_t *out_idx, cudaStream_t s) {
    const auto *sv = static_cast<const cplx_t<T> *>(svv);
    int chunk_log2 = std::max(5, int(n) - 18);
    if (chunk_log2 > int(n)) chunk_log2 = int(n);
    if (chunk_log2 < 5 && n >= 5) chunk_log2 = 5;
    const uint64_t nchunks = (uint64_t(1) << n) >> chunk_log2;
    // scratch: total (bytes 128..255) | csum, then the block offsets | draws | out
    const uint64_t nblocks = (nchunks + 1023) / 1024;  // <= 256 (nchunks <= 2^18)
    const size_t cbytes = (nchunks + nblocks) * sizeof(double);
    const size_t dbytes = shots * sizeof(double);
    const size_t obytes = shots * sizeof(uint64_t);
    void *p = nullptr;
    LGPU_TRY(ctx_scratch(ctx, 256 + ((cbytes + 255) & ~size_t(255)) + ((dbytes + 255) & ~size_t(255)) + obytes, &p));
    char *cp = static_cast<char *>(p);
    auto *total = reinterpret_cast<double *>(cp + 128);  // bytes 0..127: reduction counter, kept zero
    auto *csum = reinterpret_cast<double *>(cp + 256);
    auto *ddraws = reinterpret_cast<double *>(cp + 256 + ((cbytes + 255) & ~size_t(255)));
    auto *dout = reinterpret_cast<uint64_t *>(cp + 256 + ((cbytes + 255) & ~size_t(255)) +
                                              ((dbytes + 255) & ~size_t(255)));
    void *pin = nullptr;
    LGPU_TRY(ctx_pinned(ctx, std::max(dbytes, obytes), &pin));
    std::memcpy(pin, draws, dbytes);
    LGPU_CUDA_TRY(cudaMemcpyAsync(ddraws, pin, dbytes, cudaMemcpyHostToDevice, s));
    const unsigned g1 =
        unsigned(std::max<uint64_t>(1, std::min<uint64_t>((nchunks + 7) / 8, uint64_t(sm_count()) * 8)));
    if (n < 5) {
        // tiny states: a single chunk
        chunk_sums_kernel<T><<<1, 256, 0, s>>>(sv, 1, int(n), csum);
    } else {
        chunk_sums_kernel<T><<<g1, 256, 0, s>>>(sv, nchunks, chunk_log2, csum);
    }
    LGPU_CHECK_LAUNCH();
    const uint64_t nch = n < 5 ? 1 : nchunks;
    const int clog = n < 5 ? int(n) : chunk_log2;
    double *boff = csum + nchunks;
    const uint64_t nbl = (nch + 1023) / 1024;
    scan_blocks_kernel<<<unsigned(nbl), 1024, 0, s>>>(csum, nch, boff);
    LGPU_CHECK_LAUNCH();
    scan_tops_kernel<<<1, 32, 0, s>>>(boff, uint32_t(nbl), total);
    LGPU_CHECK_LAUNCH();
    const unsigned g2 = unsigned(std::max<uint64_t>(1, std::min<uint64_t>((shots + 7) / 8, uint64_t(sm_count()) * 8)));
    search_kernel<T><<<g2, 256, 0, s>>>(sv, csum, boff, nch, clog, total, ddraws, shots, dout);
    LGPU_CHECK_LAUNCH();
    // Copy back through the pinned buffer; the draws have already been consumed
    // by the H2D copy that precedes this D2H copy in stream order.
    LGPU_CUDA_TRY(cudaMemcpyAsync(pin, dout, obytes, cudaMemcpyDeviceToHost, s));
    LGPU_CUDA_TRY(cudaStreamSynchronize(s));
    std::memcpy(out_idx, pin, obytes);
    return LGPU_OK;
}

// ---------------------------------------------------------------------------
// Pauli sum apply: out = sum_t c_t P_t in
// ---------------------------------------------------------------------------
constexpr int kSumTerms = 16;

template <class T> struct PSumParams {
    uint64_t flip;
    int nt;
    int accumulate;
    uint64_t sgn[kSumTerms];
    double cr[kSumTerms], ci[kSumTerms];  // c_t * i^ny_t
};

template <class T>
__global__ void __launch_bounds__(256)
    pauli_sum_kernel(const cplx_t<T> *__restrict__ in, cplx_t<T> *__restrict__ out, uint64_t N, const PSumParams<T> p) {
    const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
    for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < N; i += stride) {
        const uint64_t j = i ^ p.flip;
        // (P_t in)_i = i^ny sigma_t(j) in_j
        double fr = 0, fi = 0;
        for (int t = 0; t < p.nt; t++) {
            const double sg = (__popcll(j & p.sgn[t]) & 1) ? -1.0 : 1.0;
            fr += sg * p.cr[t];
            fi += sg * p.ci[t];
        }
        const cplx_t<T> b = in[j];
        double yr = fr * double(b.x) - fi * double(b.y);
        double yi = fr * double(b.y) + fi * double(b.x);
        if (p.accumulate) {
            const cplx_t<T> o = out[i];
            yr += double(o.x);
            yi += double(o.y);
        }
        out[i] = mk<T>(T(yr), T(yi));
    }
}

// ---------------------------------------------------------------------------
// Pauli sum apply by tile passes (from 16 qubits): the words of a pass (as the
// expectation tile passes group them) flip only tile bits, so
// (sum_t c_t P_t in)_e = sum_t c_t sigma_t(e ^ flip_t) in_{e ^ flip_t} needs
// only the tile of `in`.  A CTA streams tiles of `in` through two shared-memory
// buffers; each thread forms its output elements e = tid + 256 j in registers
// over the pass's words (the source index e ^ flip = (tid ^ flip's low 8 bits)
// | ((j << 8) ^ flip's high bits), so the address is a per-thread base plus a
// per-word constant, and the sign a per-thread bit XOR a per-word constant
// bit) and adds them to `out`.  complex128 works in float-float: the tile is
// converted after its load, the products and sums run as paired lanes
// (re, im), and `out` holds float-float values (re.hi, im.hi, re.lo, im.lo)
// from the first pass to the last, then is converted back once.  complex64
// works in FP32.  Replaces one FP64-bound pass per distinct flip mask.
// ---------------------------------------------------------------------------
template <class I> struct PauliApplyParams {
    const void *in;
    void *out;
    Holes holes;
    I ntiles;
    int m, nw, accumulate;
    I hi_off[1 << kTileHiMax];
    uint32_t xlo[kTileWords];               // flip bits below bit 8 (tile positions)
    uint32_t tsign[kTileWords];             // sign mask in tile positions
    uint64_t osign[kTileWords];             // sign mask outside the tile (state bits)
    uint32_t ja[kTileWords][kPtMaxNA];      // ((j << 8) ^ flip bits from bit 8) times the element bytes
    uint32_t cs[kTileWords][kPtMaxNA];      // bit 31: parity of (((j << 8) ^ flip bits from bit 8) & sign mask)
    float c[kTileWords][4];                 // c_t i^ny_t: (re.hi, im.hi, re.lo, im.lo); complex64 (re, im, -, -)
};

template <class T, class I>
__global__ void __launch_bounds__(kPauliTileThreads, 3) pauli_apply_tile_kernel(const PauliApplyParams<I> p) {
    using Gm = PtGeom<T>;
    constexpr int E = Gm::E, NA = Gm::NA, EB = 1 << Gm::LEB;
    extern __shared__ __align__(128) unsigned char pa_smem[];
    const int tid = threadIdx.x;
    const uint32_t lowmask = (1u << p.m) - 1u;
    constexpr int EPC = sizeof(T) == 4 ? 2 : 1;   // amplitudes per 16-byte chunk
    constexpr int GEB = sizeof(T) == 4 ? 8 : 16;  // bytes per amplitude in the state
    const unsigned char *src = static_cast<const unsigned char *>(p.in);
    auto load = [&](I tau, unsigned char *dst) {
        const I base = insert_holes<I>(tau, p.holes);
        for (int c = tid; c < E / EPC; c += kPauliTileThreads) {
            const uint32_t e = uint32_t(c * EPC);
            const I gi = base + p.hi_off[e >> p.m] + I(e & lowmask);
            pt_cp_async16(dst + size_t(e) * EB, src + size_t(gi) * GEB);
        }
        asm volatile("cp.async.commit_group;" ::: "memory");
    };
    const I G = I(gridDim.x);
    I tau = blockIdx.x;
    if (tau < p.ntiles) load(tau, pa_smem);
    else asm volatile("cp.async.commit_group;" ::: "memory");
    for (int it = 0; tau < p.ntiles; tau += G, it++) {
        unsigned char *cur = pa_smem + (it & 1) * (E * EB);
        if (tau + G < p.ntiles) load(tau + G, pa_smem + ((it + 1) & 1) * (E * EB));
        else asm volatile("cp.async.commit_group;" ::: "memory");
        asm volatile("cp.async.wait_group 1;" ::: "memory");
        __syncthreads();
        if constexpr (sizeof(T) == 8) {  // complex128 -> float-float in place
#pragma unroll 4
            for (int j = 0; j < NA; j++) {
                const int e = tid + j * kPauliTileThreads;
                const double2 v = reinterpret_cast<const double2 *>(cur)[e];
                const DF r = df_from_double(v.x), im = df_from_double(v.y);
                reinterpret_cast<float4 *>(cur)[e] = make_float4(r.hi, im.hi, r.lo, im.lo);
            }
            __syncthreads();
        }
        const I base = insert_holes<I>(tau, p.holes);
        // per word: this thread's source base and sign bit for the tile
        uint32_t xb[kTileWords], ps[kTileWords];
#pragma unroll
        for (int t = 0; t < kTileWords; t++) {
            const uint32_t x = uint32_t(tid) ^ p.xlo[t];
            xb[t] = x << Gm::LEB;
            ps[t] = uint32_t(__popc(x & p.tsign[t]) + __popcll(uint64_t(base) & p.osign[t])) << 31;
        }
#pragma unroll 2
        for (int j = 0; j < NA; j++) {
            const int e = tid + j * kPauliTileThreads;
            const I gi = base + p.hi_off[uint32_t(e) >> p.m] + I(uint32_t(e) & lowmask);
            if constexpr (sizeof(T) == 4) {
                float ar = 0.0f, ai = 0.0f;
#pragma unroll
                for (int t = 0; t < kTileWords; t++) {
                    if (t >= p.nw) break;
                    const float2 x = *reinterpret_cast<const float2 *>(cur + xb[t] + p.ja[t][j]);
                    const uint32_t sb = ps[t] ^ p.cs[t][j];
                    const float xr = pt_flip_sign(x.x, sb), xi = pt_flip_sign(x.y, sb);
                    const float cr = p.c[t][0], ci = p.c[t][1];
                    ar = fmaf(cr, xr, fmaf(-ci, xi, ar));
                    ai = fmaf(cr, xi, fmaf(ci, xr, ai));
                }
                float2 *o = static_cast<float2 *>(p.out) + gi;
                if (p.accumulate) {
                    const float2 v = *o;
                    ar += v.x;
                    ai += v.y;
                }
                *o = make_float2(ar, ai);
            } else {
                DF2 acc{F2{0ull}, F2{0ull}};
#pragma unroll
                for (int t = 0; t < kTileWords; t++) {
                    if (t >= p.nw) break;
                    const float4 x = *reinterpret_cast<const float4 *>(cur + xb[t] + p.ja[t][j]);
                    const uint32_t sb = ps[t] ^ p.cs[t][j];
                    const float xr = pt_flip_sign(x.x, sb), xi = pt_flip_sign(x.y, sb);
                    const float xrl = pt_flip_sign(x.z, sb), xil = pt_flip_sign(x.w, sb);
                    const DF2 X{f2_pack(xr, xi), f2_pack(xrl, xil)}, Xs{f2_pack(xi, xr), f2_pack(xil, xrl)};
                    // (cr, cr) (xr, xi) + (-ci, ci) (xi, xr) = c x in the lanes (re, im)
                    const DF2 C1{f2_pack(p.c[t][0], p.c[t][0]), f2_pack(p.c[t][2], p.c[t][2])};
                    const DF2 C2{f2_pack(-p.c[t][1], p.c[t][1]), f2_pack(-p.c[t][3], p.c[t][3])};
                    acc = df2_sum<3>({acc, df2_mul(C1, X), df2_mul(C2, Xs)});
                }
                float4 *o = static_cast<float4 *>(p.out) + gi;
                if (p.accumulate) {
                    const float4 v = *o;
                    acc = df2_sum<2>({acc, DF2{f2_pack(v.x, v.y), f2_pack(v.z, v.w)}});
                }
                *o = make_float4(f2_x(acc.hi), f2_y(acc.hi), f2_x(acc.lo), f2_y(acc.lo));
            }
        }
        __syncthreads();  // `cur` is the target of a load issued next iteration
    }
    asm volatile("cp.async.wait_group 0;" ::: "memory");
}

// out (float-float, (re.hi, im.hi, re.lo, im.lo) per amplitude) -> complex128, in place.
__global__ void __launch_bounds__(256) ff_to_c128_kernel(double2 *sv, uint64_t count) {
    const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
    for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < count; i += stride) {
        const float4 v = reinterpret_cast<const float4 *>(sv)[i];
        sv[i] = make_double2(df_to_double(DF{v.x, v.z}), df_to_double(DF{v.y, v.w}));
    }
}

// The terms whose flips fit a tile, by tile passes; done[w] = 1 for those.
// `out` ends as complex128 (the first pass overwrites it).
template <class T, class I>
static lgpu_status_t pauli_apply_tiles(const void *in, void *out, uint32_t n, uint32_t nterms, const double *coeffs,
                                       const uint64_t *flip, const uint64_t *sign, const uint8_t *ny,
                                       std::vector<char> &done, cudaStream_t s) {
    using Gm = PtGeom<T>;
    done.assign(nterms, 0);
    if (n < uint32_t(Gm::K)) return LGPU_OK;
    const auto passes = plan_tile_passes(n, nterms, flip, Gm::K, Gm::MMIN);
    if (passes.empty()) return LGPU_OK;
    const unsigned grid_cap = unsigned(sm_count()) * 3;
    static std::atomic<size_t> attr[64];
    const size_t smem = 2 * size_t(Gm::E) * (size_t(1) << Gm::LEB);
    LGPU_TRY(ensure_smem(reinterpret_cast<const void *>(pauli_apply_tile_kernel<T, I>), smem, attr));
    for (size_t pi = 0; pi < passes.size(); pi++) {
        const TilePass &tp = passes[pi];
        const int k = int(tp.tile.size());
        if (k != Gm::K) return fail(LGPU_ERR_UNSUPPORTED, "Pauli tile pass of unexpected size");
        int m = 0;
        while (m < k && tp.tile[size_t(m)] == m) m++;
        auto b = std::make_unique<PauliApplyParams<I>>();
        std::memset(b.get(), 0, sizeof(PauliApplyParams<I>));
        b->in = in;
        b->out = out;
        b->holes = make_holes(tp.tile);
        b->ntiles = I(uint64_t(1) << (n - uint32_t(k)));
        b->m = m;
        b->nw = int(tp.words.size());
        b->accumulate = pi > 0 ? 1 : 0;
        for (int h = 0; h < (1 << (k - m)); h++) {
            uint64_t o = 0;
            for (int q = m; q < k; q++)
                if ((h >> (q - m)) & 1) o |= uint64_t(1) << tp.tile[size_t(q)];
            b->hi_off[h] = I(o);
        }
        for (int t = 0; t < b->nw; t++) {
            const uint32_t w = tp.words[size_t(t)];
            uint32_t tf = 0, ts = 0;
            uint64_t os = sign[w];
            for (int q = 0; q < k; q++) {
                const int bit = tp.tile[size_t(q)];
                if ((flip[w] >> bit) & 1u) tf |= 1u << q;
                if ((sign[w] >> bit) & 1u) {
                    ts |= 1u << q;
                    os &= ~(uint64_t(1) << bit);
                }
            }
            b->xlo[t] = tf & 0xFFu;
            b->tsign[t] = ts;
            b->osign[t] = os;
            for (int j = 0; j < Gm::NA; j++) {
                const uint32_t J = (uint32_t(j) << 8) ^ (tf & ~0xFFu);
                b->ja[t][j] = J << Gm::LEB;
                b->cs[t][j] = uint32_t(__builtin_popcount(J & ts) & 1) << 31;
            }
            double cr = coeffs[2 * w], ci = coeffs[2 * w + 1];
            for (int q = 0; q < (ny[w] & 3); q++) {  // multiply by i
                const double tr = -ci;
                ci = cr;
                cr = tr;
            }
            if (sizeof(T) == 8) {
                const DF r = df_split_host(cr), i = df_split_host(ci);
                b->c[t][0] = r.hi;
                b->c[t][1] = i.hi;
                b->c[t][2] = r.lo;
                b->c[t][3] = i.lo;
            } else {
                b->c[t][0] = float(cr);
                b->c[t][1] = float(ci);
            }
            done[w] = 1;
        }
        const unsigned grid = unsigned(std::min<uint64_t>(uint64_t(b->ntiles), grid_cap));
        pauli_apply_tile_kernel<T, I><<<grid, kPauliTileThreads, smem, s>>>(*b);
        LGPU_CHECK_LAUNCH();
    }
    if (sizeof(T) == 8) {
        const uint64_t count = uint64_t(1) << n;
        ff_to_c128_kernel<<<grid_for(count, 256, 8, 8), 256, 0, s>>>(static_cast<double2 *>(out), count);
        LGPU_CHECK_LAUNCH();
    }
    return LGPU_OK;
}

template <class T>
static lgpu_status_t pauli_sum_t(const void *in, void *out, uint32_t n, uint32_t nterms, const double *coeffs,
                                 const uint64_t *flip, const uint64_t *sign, const uint8_t *ny, cudaStream_t s) {
    std::vector<uint64_t> keys;
    std::vector<std::vector<uint32_t>> groups;
    for (uint32_t w = 0; w < nterms; w++) {
        size_t gi = 0;
        for (; gi < keys.size(); gi++)
            if (keys[gi] == flip[w]) break;
        if (gi == keys.size()) {
            keys.push_back(flip[w]);
            groups.emplace_back();
        }
        groups[gi].push_back(w);
    }
    const uint64_t N = uint64_t(1) << n;
    bool first = true;
    if (nterms == 0) {
        LGPU_CUDA_TRY(cudaMemsetAsync(out, 0, N * sizeof(cplx_t<T>), s));
        return LGPU_OK;
    }
    // from 16 qubits the terms whose flips fit a tile go through tile passes
    // (float-float / FP32); the rest add to `out` one pass per flip mask
    std::vector<char> done(nterms, 0);
    if (n >= 16) {
        const lgpu_status_t st = n <= 32
                                     ? pauli_apply_tiles<T, uint32_t>(in, out, n, nterms, coeffs, flip, sign, ny, done, s)
                                     : pauli_apply_tiles<T, uint64_t>(in, out, n, nterms, coeffs, flip, sign, ny, done, s);
        LGPU_TRY(st);
        for (uint32_t w = 0; w < nterms; w++)
            if (done[w]) {
                first = false;
                break;
            }
    }
    for (size_t gi = 0; gi < keys.size(); gi++) {
        auto &gw = groups[gi];
        gw.erase(std::remove_if(gw.begin(), gw.end(), [&](uint32_t w) { return done[w] != 0; }), gw.end());
        for (size_t o = 0; o < groups[gi].size(); o += kSumTerms) {
            PSumParams<T> p{};
            p.flip = keys[gi];
            p.accumulate = first ? 0 : 1;
            first = false;
            p.nt = int(std::min<size_t>(kSumTerms, groups[gi].size() - o));
            for (int t = 0; t < p.nt; t++) {
                const uint32_t w = groups[gi][o + size_t(t)];
                p.sgn[t] = sign[w];
                double cr = coeffs[2 * w], ci = coeffs[2 * w + 1];
                for (int q = 0; q < (ny[w] & 3); q++) {  // multiply by i
                    const double tr = -ci;
                    ci = cr;
                    cr = tr;
                }
                p.cr[t] = cr;
                p.ci[t] = ci;
            }
            pauli_sum_kernel<T><<<grid_for(N, 256, 4), 256, 0, s>>>(static_cast<const cplx_t<T> *>(in),
                                                                    static_cast<cplx_t<T> *>(out), N, p);
            LGPU_CHECK_LAUNCH();
        }
    }
    return LGPU_OK;
}

// ---------------------------------------------------------------------------
// CSR
// ---------------------------------------------------------------------------
template <class T>
__global__ void spmv_kernel(const int64_t *__restrict__ off, const int64_t *__restrict__ cols,
                            const cplx_t<T> *__restrict__ vals, const cplx_t<T> *__restrict__ x, cplx_t<T> *y,
                            uint64_t nrows) {
    const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
    for (uint64_t r = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; r < nrows; r += stride) {
        double ar = 0, ai = 0;
        for (int64_t q = off[r]; q < off[r + 1]; q++) {
            const cplx_t<T> v = vals[q], b = x[cols[q]];
            ar += double(v.x) * b.x - double(v.y) * b.y;
            ai += double(v.x) * b.y + double(v.y) * b.x;
        }
        y[r] = mk<T>(T(ar), T(ai));
    }
}

template <class T> struct CsrExpBody {
    const int64_t *off;
    const int64_t *cols;
    const cplx_t<T> *vals;
    const cplx_t<T> *x;
    __device__ __forceinline__ void operator()(uint64_t r, double2 *acc) const {
        double ar = 0, ai = 0;
        for (int64_t q = off[r]; q < off[r + 1]; q++) {
            const cplx_t<T> v = vals[q], b = x[cols[q]];
            ar += double(v.x) * b.x - double(v.y) * b.y;
            ai += double(v.x) * b.y + double(v.y) * b.x;
        }
        const cplx_t<T> a = x[r];
        acc[0].x += double(a.x) * ar + double(a.y) * ai;
        acc[0].y += double(a.x) * ai - double(a.y) * ar;
    }
};

}  // namespace lgpu

using namespace lgpu;

extern "C" {

lgpu_status_t lgpu_expval_matrix(lgpu_context_t ctx, const void *sv, uint32_t n, lgpu_dtype_t dt,
                                 const double *matrix, uint32_t t, const int32_t *tgts, double *out,
                                 int out_on_device, lgpu_stream_t stream) {
    LGPU_TRY(check_state(sv, n, dt));
    if (!matrix || !out) return fail(LGPU_ERR_INVALID_ARG, "null matrix/output");
    if (t < 1 || t > LGPU_MAX_EXPVAL_TARGETS || t > n)
        return fail(LGPU_ERR_INVALID_ARG, "expval: number of targets must be in [1, " +
                                              std::to_string(LGPU_MAX_EXPVAL_TARGETS) + "] and at most n");
    std::vector<int> tg;
    LGPU_TRY(check_bits(n, t, tgts, "target", &tg));
    std::vector<int> srt(tg);
    std::sort(srt.begin(), srt.end());
    if (std::adjacent_find(srt.begin(), srt.end()) != srt.end())
        return fail(LGPU_ERR_INVALID_ARG, "repeated target bit");
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    if (dt == LGPU_C128)
        return n <= 32 ? expval_dispatch<double, uint32_t>(ctx, sv, n, matrix, tg, out, out_on_device, s)
                       : expval_dispatch<double, uint64_t>(ctx, sv, n, matrix, tg, out, out_on_device, s);
    return n <= 32 ? expval_dispatch<float, uint32_t>(ctx, sv, n, matrix, tg, out, out_on_device, s)
                   : expval_dispatch<float, uint64_t>(ctx, sv, n, matrix, tg, out, out_on_device, s);
}

lgpu_status_t lgpu_expval_pauli_words(lgpu_context_t ctx, const void *sv, uint32_t n, lgpu_dtype_t dt,
                                      uint32_t nwords, const uint64_t *flip, const uint64_t *sign,
                                      const uint8_t *ny, double *out, int out_on_device, lgpu_stream_t stream) {
    LGPU_TRY(check_state(sv, n, dt));
    if (nwords == 0) return LGPU_OK;
    if (!flip || !sign || !ny || !out) return fail(LGPU_ERR_INVALID_ARG, "null argument");
    const uint64_t full = n >= 64 ? ~uint64_t(0) : ((uint64_t(1) << n) - 1);
    for (uint32_t w = 0; w < nwords; w++)
        if ((flip[w] | sign[w]) & ~full) return fail(LGPU_ERR_INVALID_ARG, "Pauli word mask exceeds the qubit count");
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    if (dt == LGPU_C128)
        return n <= 32 ? pauli_words_t<double, uint32_t>(ctx, sv, n, nwords, flip, sign, ny, out, out_on_device, s)
                       : pauli_words_t<double, uint64_t>(ctx, sv, n, nwords, flip, sign, ny, out, out_on_device, s);
    return n <= 32 ? pauli_words_t<float, uint32_t>(ctx, sv, n, nwords, flip, sign, ny, out, out_on_device, s)
                   : pauli_words_t<float, uint64_t>(ctx, sv, n, nwords, flip, sign, ny, out, out_on_device, s);
}

lgpu_status_t lgpu_probs(lgpu_context_t ctx, const void *sv, uint32_t n, lgpu_dtype_t dt, uint32_t k,
                         const int32_t *bits, double *out, int out_on_device, lgpu_stream_t stream) {
    LGPU_TRY(check_state(sv, n, dt));
    if (!out) return fail(LGPU_ERR_INVALID_ARG, "output is null");
    if (k > 24 || k > n) return fail(LGPU_ERR_INVALID_ARG, "probs: at most 24 bits");
    std::vector<int> b;
    LGPU_TRY(check_bits(n, k, bits, "probability", &b));
    std::vector<int> srt(b);
    std::sort(srt.begin(), srt.end());
    if (std::adjacent_find(srt.begin(), srt.end()) != srt.end())
        return fail(LGPU_ERR_INVALID_ARG, "repeated probability bit");
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    if (dt == LGPU_C128)
        return n <= 32 ? probs_t<double, uint32_t>(ctx, sv, n, b, out, out_on_device, s)
                       : probs_t<double, uint64_t>(ctx, sv, n, b, out, out_on_device, s);
    return n <= 32 ? probs_t<float, uint32_t>(ctx, sv, n, b, out, out_on_device, s)
                   : probs_t<float, uint64_t>(ctx, sv, n, b, out, out_on_device, s);
}

lgpu_status_t lgpu_sample(lgpu_context_t ctx, const void *sv, uint32_t n, lgpu_dtype_t dt, const double *draws,
                          uint64_t shots, uint64_t *out_idx, lgpu_stream_t stream) {
    LGPU_TRY(check_state(sv, n, dt));
    if (shots == 0) return LGPU_OK;
    if (!draws || !out_idx) return fail(LGPU_ERR_INVALID_ARG, "null draws/output");
    for (uint64_t i = 0; i < shots; i++)
        if (!(draws[i] >= 0.0 && draws[i] < 1.0)) return fail(LGPU_ERR_INVALID_ARG, "draws must lie in [0, 1)");
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    return dt == LGPU_C128 ? sample_t<double>(ctx, sv, n, draws, shots, out_idx, s)
                           : sample_t<float>(ctx, sv, n, draws, shots, out_idx, s);
}

lgpu_status_t lgpu_apply_pauli_sum(const void *in, void *out, uint32_t n, lgpu_dtype_t dt, uint32_t nterms,
                                   const double *coeffs, const uint64_t *flip, const uint64_t *sign,
                                   const uint8_t *ny, lgpu_stream_t stream) {
    LGPU_TRY(check_state(in, n, dt));
    LGPU_TRY(check_state(out, n, dt));
    if (in == out) return fail(LGPU_ERR_INVALID_ARG, "pauli sum: in and out must not alias");
    if (nterms && (!coeffs || !flip || !sign || !ny)) return fail(LGPU_ERR_INVALID_ARG, "null argument");
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    return dt == LGPU_C128 ? pauli_sum_t<double>(in, out, n, nterms, coeffs, flip, sign, ny, s)
                           : pauli_sum_t<float>(in, out, n, nterms, coeffs, flip, sign, ny, s);
}

lgpu_status_t lgpu_spmv_csr(const int64_t *offsets, const int64_t *cols, const void *vals, const void *x, void *y,
                            uint32_t n, lgpu_dtype_t dt, lgpu_stream_t stream) {
    LGPU_TRY(check_state(x, n, dt));
    LGPU_TRY(check_state(y, n, dt));
    if (!offsets || !cols || !vals) return fail(LGPU_ERR_INVALID_ARG, "null CSR array");
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const uint64_t N = uint64_t(1) << n;
    if (dt == LGPU_C128)
        spmv_kernel<double><<<grid_for(N, 256, 1), 256, 0, s>>>(offsets, cols, static_cast<const double2 *>(vals),
                                                                static_cast<const double2 *>(x),
                                                                static_cast<double2 *>(y), N);
    else
        spmv_kernel<float><<<grid_for(N, 256, 1), 256, 0, s>>>(offsets, cols, static_cast<const float2 *>(vals),
                                                               static_cast<const float2 *>(x),
                                                               static_cast<float2 *>(y), N);
    LGPU_CHECK_LAUNCH();
    return LGPU_OK;
}

lgpu_status_t lgpu_expval_csr(lgpu_context_t ctx, const int64_t *offsets, const int64_t *cols, const void *vals,
                              const void *x, uint32_t n, lgpu_dtype_t dt, double *out, int out_on_device,
                              lgpu_stream_t stream) {
    LGPU_TRY(check_state(x, n, dt));
    if (!offsets || !cols || !vals || !out) return fail(LGPU_ERR_INVALID_ARG, "null argument");
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const uint64_t N = uint64_t(1) << n;
    const unsigned g = reduce_grid(N);
    ReduceScratch rs;
    LGPU_TRY(reduce_scratch(ctx, g, 1, &rs));
    double2 *res = rs.partials + size_t(g);
    if (dt == LGPU_C128) {
        CsrExpBody<double> b{offsets, cols, static_cast<const double2 *>(vals), static_cast<const double2 *>(x)};
        reduce_kernel<1, uint64_t><<<g, kReduceBlock, 0, s>>>(b, N, rs.partials, rs.counter, res);
    } else {
        CsrExpBody<float> b{offsets, cols, static_cast<const float2 *>(vals), static_cast<const float2 *>(x)};
        reduce_kernel<1, uint64_t><<<g, kReduceBlock, 0, s>>>(b, N, rs.partials, rs.counter, res);
    }
    LGPU_CHECK_LAUNCH();
    return deliver(ctx, res, 1, out, out_on_device, s);
}

}  // extern "C"
