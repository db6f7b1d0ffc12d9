// liblgpu_gb300: one fused step of the adjoint-Jacobian reverse sweep.
//
// For an operation U acting on the bit set `bits` (w <= 4 bits, controls
// folded into a block matrix) with generator G on the same bits, one launch
// streams the ket and up to 8 bras once:
//     out[k] = Im <bra_k| G |ket>           (pre-update values)
//     bra_k <- U^dag bra_k ;  ket <- U^dag ket   (optional)
// which replaces the reference's per-op sequence of a D2D copy of lambda,
// U^dag on lambda, G on mu, K cuBLAS dot products and U^dag on K bras
// (AdjointDiffGPU.hpp:560-595).
#include <algorithm>
#include <complex>
#include <cstddef>
#include <memory>
#include <vector>

#include "lgpu_adj_plan.h"
#include "lgpu_bodies.cuh"
#include "lgpu_df2.cuh"
#include "lgpu_df64.cuh"
#include "lgpu_internal.cuh"
#include "lgpu_reduce.cuh"

namespace lgpu {

constexpr int kAdjBras = 8;

template <class T, class I, int W> struct AdjBody {
    static constexpr int D = 1 << W;
    Holes holes;
    I off[D];
    double g[2 * D * D];
    double u[2 * D * D];
    int has_g;
    int apply_u;
    int update_ket;
    int nb;
    cplx_t<T> *ket;
    cplx_t<T> *bras[kAdjBras];

    __device__ __forceinline__ void matvec(const double *m, const double *xr, const double *xi, double *yr,
                                           double *yi) const {
#pragma unroll
        for (int r = 0; r < D; r++) {
            double ar = 0, ai = 0;
#pragma unroll
            for (int c = 0; c < D; c++) {
                const double mr = m[2 * (r * D + c)], mi = m[2 * (r * D + c) + 1];
                ar = fma(mr, xr[c], fma(-mi, xi[c], ar));
                ai = fma(mr, xi[c], fma(mi, xr[c], ai));
            }
            yr[r] = ar;
            yi[r] = ai;
        }
    }

    __device__ __forceinline__ void operator()(I gidx, double2 *acc) const {
        const I base = insert_holes<I>(gidx, holes);
        double kr[D], ki[D], yr[D], yi[D];
#pragma unroll
        for (int c = 0; c < D; c++) {
            const cplx_t<T> v = ket[base | off[c]];
            kr[c] = double(v.x);
            ki[c] = double(v.y);
        }
        if (has_g) matvec(g, kr, ki, yr, yi);
#pragma unroll 1
        for (int b = 0; b < nb; b++) {
            cplx_t<T> *bp = bras[b];
            double br[D], bi[D];
#pragma unroll
            for (int c = 0; c < D; c++) {
                const cplx_t<T> v = bp[base | off[c]];
                br[c] = double(v.x);
                bi[c] = double(v.y);
            }
            if (has_g) {
                double im = 0;
#pragma unroll
                for (int r = 0; r < D; r++) im = fma(br[r], yi[r], fma(-bi[r], yr[r], im));
                // acc[b] is selected by a uniform loop index: keep it in registers
#pragma unroll
                for (int q = 0; q < kAdjBras; q++)
                    if (q == b) acc[q].x += im;
            }
            if (apply_u) {
                double zr[D], zi[D];
                matvec(u, br, bi, zr, zi);
#pragma unroll
                for (int r = 0; r < D; r++) bp[base | off[r]] = mk<T>(T(zr[r]), T(zi[r]));
            }
        }
        if (update_ket) {
            matvec(u, kr, ki, yr, yi);
#pragma unroll
            for (int r = 0; r < D; r++) ket[base | off[r]] = mk<T>(T(yr[r]), T(yi[r]));
        }
    }
};

// One-bit operations (every rotation, PhaseShift and fixed 1-qubit gate):
// U^dag runs the structured 1-target bodies (integer-pipe multiplies for
// complex128) and the generator expectation has closed forms for the
// generators the named gates have, in the state's precision per pair:
//   Z: Im(b0* k0 - b1* k1)   X: Im(b0* k1 + b1* k0)
//   Y: Re(b1* k0) - Re(b0* k1)   P1 = |1><1|: Im(b1* k1)
// instead of two dense FP64 2x2 products per bra and pair.
enum GenKind : int { G_NONE = 0, G_X, G_Y, G_Z, G_P1, G_DENSE };

// GK / UB fix the generator kind and the U^dag body at compile time for the
// pairs the named rotations produce; -1 selects them at run time.  (Small
// run-time switches inside the per-pair loop are if-converted by the
// compiler, which then issues every case's FP64 work for every pair.)
template <class T, class I, bool EMU, int GK = -1, int UB = -1> struct Adj1Body {
    Holes holes;
    I tbit;
    int gk;
    int ub;  // Body1 of U^dag
    int apply_u;
    int update_ket;
    int nb;
    T g[8];  // dense generator (G_DENSE)
    T m[8];  // U^dag
    KConst k[4];
    cplx_t<T> *ket;
    cplx_t<T> *bras[kAdjBras];

    __device__ __forceinline__ T gexp(const cplx_t<T> &b0, const cplx_t<T> &b1, const cplx_t<T> &k0,
                                      const cplx_t<T> &k1) const {
        if constexpr (GK == G_Z) return (b0.x * k0.y - b0.y * k0.x) - (b1.x * k1.y - b1.y * k1.x);
        if constexpr (GK == G_X) return (b0.x * k1.y - b0.y * k1.x) + (b1.x * k0.y - b1.y * k0.x);
        if constexpr (GK == G_Y) return (b1.x * k0.x + b1.y * k0.y) - (b0.x * k1.x + b0.y * k1.y);
        if constexpr (GK == G_P1) return b1.x * k1.y - b1.y * k1.x;
        switch (gk) {
        case G_Z: return (b0.x * k0.y - b0.y * k0.x) - (b1.x * k1.y - b1.y * k1.x);
        case G_X: return (b0.x * k1.y - b0.y * k1.x) + (b1.x * k0.y - b1.y * k0.x);
        case G_Y: return (b1.x * k0.x + b1.y * k0.y) - (b0.x * k1.x + b0.y * k1.y);
        case G_P1: return b1.x * k1.y - b1.y * k1.x;
        default: {
            // (G k)_r then Im(b_r* (G k)_r)
            const T y0r = g[0] * k0.x - g[1] * k0.y + g[2] * k1.x - g[3] * k1.y;
            const T y0i = g[0] * k0.y + g[1] * k0.x + g[2] * k1.y + g[3] * k1.x;
            const T y1r = g[4] * k0.x - g[5] * k0.y + g[6] * k1.x - g[7] * k1.y;
            const T y1i = g[4] * k0.y + g[5] * k0.x + g[6] * k1.y + g[7] * k1.x;
            return (b0.x * y0i - b0.y * y0r) + (b1.x * y1i - b1.y * y1r);
        }
        }
    }

    __device__ __forceinline__ void udag(cplx_t<T> &a0, cplx_t<T> &a1) const {
        if constexpr (UB >= 0) {
            body1_sel<T, (UB >= 0 ? UB : 0), EMU>(m, k, a0, a1);
            return;
        }
        switch (ub) {
        case B_DIAG: body1_sel<T, B_DIAG, EMU>(m, k, a0, a1); break;
        case B_PERM: body1_sel<T, B_PERM, EMU>(m, k, a0, a1); break;
        case B_ANTIDIAG: body1_sel<T, B_ANTIDIAG, EMU>(m, k, a0, a1); break;
        case B_REAL: body1_sel<T, B_REAL, EMU>(m, k, a0, a1); break;
        case B_RXLIKE: body1_sel<T, B_RXLIKE, EMU>(m, k, a0, a1); break;
        default: body1_sel<T, B_DENSE, EMU>(m, k, a0, a1); break;
        }
    }

    __device__ __forceinline__ void operator()(I gidx, double2 *acc) const {
        const I i0 = insert_holes<I>(gidx, holes), i1 = i0 | tbit;
        cplx_t<T> k0 = ket[i0], k1 = ket[i1];
        // compile-time bra index: acc[b] stays a register (a runtime index
        // would cost an FP64 add per accumulator slot)
#pragma unroll
        for (int b = 0; b < kAdjBras; b++) {
            if (b >= nb) break;
            cplx_t<T> *bp = bras[b];
            cplx_t<T> b0 = bp[i0], b1 = bp[i1];
            if (GK >= 0 || gk != G_NONE) acc[b].x += double(gexp(b0, b1, k0, k1));
            if (apply_u) {
                udag(b0, b1);
                bp[i0] = b0;
                bp[i1] = b1;
            }
        }
        if (update_ket) {
            udag(k0, k1);
            ket[i0] = k0;
            ket[i1] = k1;
        }
    }
};

// Exact classification of a 2x2 generator (re/im interleaved).
static int gen_kind(const double *g) {
    auto is = [&](int e, double re, double im) { return g[2 * e] == re && g[2 * e + 1] == im; };
    if (is(0, 1, 0) && is(1, 0, 0) && is(2, 0, 0) && is(3, -1, 0)) return G_Z;
    if (is(0, 0, 0) && is(1, 1, 0) && is(2, 1, 0) && is(3, 0, 0)) return G_X;
    if (is(0, 0, 0) && is(1, 0, -1) && is(2, 0, 1) && is(3, 0, 0)) return G_Y;
    if (is(0, 0, 0) && is(1, 0, 0) && is(2, 0, 0) && is(3, 1, 0)) return G_P1;
    return G_DENSE;
}

template <class T, class I, bool EMU, int GK, int UB>
static lgpu_status_t adjoint1_launch(lgpu_context_t ctx, void *ket, void *const *bras, uint32_t nbras, uint32_t n,
                                     int bit, const double *gen, const double *udag, int apply_udag, double *out_dev,
                                     cudaStream_t s);

template <class T, class I, bool EMU>
static lgpu_status_t adjoint1_t(lgpu_context_t ctx, void *ket, void *const *bras, uint32_t nbras, uint32_t n, int bit,
                                const double *gen, const double *udag, int apply_udag, double *out_dev, cudaStream_t s) {
    const int gk = gen ? gen_kind(gen) : G_NONE;
    KConst kc[4];
    const int ub = udag ? body_of_2x2_host(udag, kc) : B_DENSE;
    if (gk == G_X && ub == B_RXLIKE)
        return adjoint1_launch<T, I, EMU, G_X, B_RXLIKE>(ctx, ket, bras, nbras, n, bit, gen, udag, apply_udag, out_dev, s);
    if (gk == G_Y && ub == B_REAL)
        return adjoint1_launch<T, I, EMU, G_Y, B_REAL>(ctx, ket, bras, nbras, n, bit, gen, udag, apply_udag, out_dev, s);
    if (gk == G_Z && ub == B_DIAG)
        return adjoint1_launch<T, I, EMU, G_Z, B_DIAG>(ctx, ket, bras, nbras, n, bit, gen, udag, apply_udag, out_dev, s);
    if (gk == G_P1 && ub == B_DIAG)
        return adjoint1_launch<T, I, EMU, G_P1, B_DIAG>(ctx, ket, bras, nbras, n, bit, gen, udag, apply_udag, out_dev, s);
    return adjoint1_launch<T, I, EMU, -1, -1>(ctx, ket, bras, nbras, n, bit, gen, udag, apply_udag, out_dev, s);
}

template <class T, class I, bool EMU, int GK, int UB>
static lgpu_status_t adjoint1_launch(lgpu_context_t ctx, void *ket, void *const *bras, uint32_t nbras, uint32_t n,
                                     int bit, const double *gen, const double *udag, int apply_udag, double *out_dev,
                                     cudaStream_t s) {
    Adj1Body<T, I, EMU, GK, UB> b{};
    b.holes = make_holes(std::vector<int>{bit});
    b.tbit = I(I(1) << bit);
    b.gk = gen ? gen_kind(gen) : G_NONE;
    if (gen)
        for (int e = 0; e < 8; e++) b.g[e] = T(gen[e]);
    b.ub = B_DENSE;
    if (udag) {
        KConst kc[4];
        b.ub = body_of_2x2_host(udag, kc);
        for (int e = 0; e < 8; e++) b.m[e] = T(udag[e]);
        for (int e = 0; e < 4; e++) b.k[e] = kc[e];
    }
    b.ket = static_cast<cplx_t<T> *>(ket);
    const I ngroups = I(uint64_t(1) << (n - 1));
    // FP64/FP32 work per pair is a few dozen operations per bra: spread the
    // pairs thinly (one per thread) so small states still use many SMs
    const unsigned g = grid_for(uint64_t(ngroups), kReduceBlock, 1, 4);
    ReduceScratch rs;
    LGPU_TRY(reduce_scratch(ctx, g, kAdjBras, &rs));
    double2 *res = rs.partials + size_t(g) * kAdjBras;
    const uint32_t nchunks = nbras == 0 ? 1 : (nbras + kAdjBras - 1) / kAdjBras;
    for (uint32_t ch = 0; ch < nchunks; ch++) {
        const uint32_t lo = ch * kAdjBras;
        const uint32_t cnt = nbras == 0 ? 0 : std::min<uint32_t>(kAdjBras, nbras - lo);
        b.nb = int(cnt);
        for (uint32_t q = 0; q < kAdjBras; q++)
            b.bras[q] = q < cnt ? static_cast<cplx_t<T> *>(bras[lo + q]) : nullptr;
        b.apply_u = apply_udag && udag ? 1 : 0;
        b.update_ket = (apply_udag && udag && ch + 1 == nchunks) ? 1 : 0;
        reduce_kernel<kAdjBras, I><<<g, kReduceBlock, 0, s>>>(b, ngroups, rs.partials, rs.counter, res);
        LGPU_CHECK_LAUNCH();
        if (gen && cnt)
            LGPU_CUDA_TRY(cudaMemcpy2DAsync(out_dev + lo, sizeof(double), res, sizeof(double2), sizeof(double), cnt,
                                            cudaMemcpyDeviceToDevice, s));
    }
    return LGPU_OK;
}

template <class T, class I, int W>
static lgpu_status_t adjoint_t(lgpu_context_t ctx, void *ket, void *const *bras, uint32_t nbras, uint32_t n,
                               const std::vector<int> &bits, const double *gen, const double *udag, int apply_udag,
                               double *out_dev, cudaStream_t s) {
    constexpr int D = 1 << W;
    auto *b = new AdjBody<T, I, W>();
    b->holes = make_holes(bits);
    for (int r = 0; r < D; r++) {
        uint64_t o = 0;
        for (int k = 0; k < W; k++)
            if ((r >> (W - 1 - k)) & 1) o |= uint64_t(1) << bits[size_t(k)];
        b->off[r] = I(o);
    }
    b->has_g = gen ? 1 : 0;
    if (gen) std::memcpy(b->g, gen, sizeof(double) * 2 * D * D);
    if (udag) std::memcpy(b->u, udag, sizeof(double) * 2 * D * D);
    b->ket = static_cast<cplx_t<T> *>(ket);
    const I ngroups = I(uint64_t(1) << (n - W));
    // dense FP64 products per group: one group per thread
    const unsigned g = grid_for(uint64_t(ngroups), kReduceBlock, 1, 4);
    ReduceScratch rs;
    lgpu_status_t st = reduce_scratch(ctx, g, kAdjBras, &rs);
    if (st != LGPU_OK) {
        delete b;
        return st;
    }
    double2 *res = rs.partials + size_t(g) * kAdjBras;
    const uint32_t nchunks = nbras == 0 ? 1 : (nbras + kAdjBras - 1) / kAdjBras;
    for (uint32_t ch = 0; ch < nchunks; ch++) {
        const uint32_t lo = ch * kAdjBras;
        const uint32_t cnt = nbras == 0 ? 0 : std::min<uint32_t>(kAdjBras, nbras - lo);
        b->nb = int(cnt);
        for (uint32_t q = 0; q < cnt; q++) b->bras[q] = static_cast<cplx_t<T> *>(bras[lo + q]);
        b->apply_u = apply_udag && udag ? 1 : 0;
        b->update_ket = (apply_udag && udag && ch + 1 == nchunks) ? 1 : 0;
        reduce_kernel<kAdjBras, I><<<g, kReduceBlock, 0, s>>>(*b, ngroups, rs.partials, rs.counter, res);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) {
            delete b;
            return cuda_fail(e, "adjoint step launch");
        }
        if (gen && cnt) {
            // out_dev[lo + q] = res[q].x  (strided copy of the real parts)
            e = cudaMemcpy2DAsync(out_dev + lo, sizeof(double), res, sizeof(double2), sizeof(double), cnt,
                                  cudaMemcpyDeviceToDevice, s);
            if (e != cudaSuccess) {
                delete b;
                return cuda_fail(e, "adjoint result copy");
            }
        }
    }
    delete b;
    return LGPU_OK;
}

template <class T, class I>
static lgpu_status_t adjoint_dispatch(lgpu_context_t ctx, void *ket, void *const *bras, uint32_t nbras, uint32_t n,
                                      const std::vector<int> &bits, const double *gen, const double *udag,
                                      int apply_udag, double *out_dev, cudaStream_t s) {
    switch (bits.size()) {
    case 1:
        if constexpr (sizeof(T) == 8)
            return f64_mode() == 1
                       ? adjoint1_t<T, I, true>(ctx, ket, bras, nbras, n, bits[0], gen, udag, apply_udag, out_dev, s)
                       : adjoint1_t<T, I, false>(ctx, ket, bras, nbras, n, bits[0], gen, udag, apply_udag, out_dev, s);
        else
            return adjoint1_t<T, I, false>(ctx, ket, bras, nbras, n, bits[0], gen, udag, apply_udag, out_dev, s);
    case 2: return adjoint_t<T, I, 2>(ctx, ket, bras, nbras, n, bits, gen, udag, apply_udag, out_dev, s);
    case 3: return adjoint_t<T, I, 3>(ctx, ket, bras, nbras, n, bits, gen, udag, apply_udag, out_dev, s);
    case 4: return adjoint_t<T, I, 4>(ctx, ket, bras, nbras, n, bits, gen, udag, apply_udag, out_dev, s);
    default: return fail(LGPU_ERR_INVALID_ARG, "adjoint step: 1 to 4 bits");
    }
}

// ---------------------------------------------------------------------------
// Whole reverse sweep in shared memory (small states)
// ---------------------------------------------------------------------------
// One CTA per bra: lambda and the bra live in shared memory for the whole
// sweep, so a 12-qubit circuit of a few hundred operations is one launch
// instead of a few hundred.  U^dag runs as a 1-target structured body under
// controls (every named 1- and 2-qubit gate but SWAP and the Ising family,
// which run as dense 4x4), the generator expectation in closed form for
// X, Y, Z and |1><1| (also under one control, as for CRX/CRY/CRZ/CPhase).
constexpr int kSweepThreads = 512;
enum UKind : int { U_NONE = 0, U_ONE = 1, U_DENSE4 = 2 };

struct SweepOp {
    int ukind, ubody, ut, uq2;  // U_ONE: body on bit ut under (ucm, ucv); U_DENSE4: (ut, uq2), ut = matrix MSB
    uint32_t ucm, ucv;
    int gkind, gt, gq2;         // G_X..G_DENSE on gt under (gcm, gcv); G_DENSE4 on (gt, gq2)
    uint32_t gcm, gcv;
    int col;
    double u[32];
    double g[32];
    float uf[32];
    float gf[32];
    KConst uk[4];
};
constexpr int G_DENSE4 = 16;

template <class T> __device__ __forceinline__ const T *op_u(const SweepOp &o) {
    if constexpr (sizeof(T) == 4) return o.uf;
    else return o.u;
}
template <class T> __device__ __forceinline__ const T *op_g(const SweepOp &o) {
    if constexpr (sizeof(T) == 4) return o.gf;
    else return o.g;
}

// One 1-target body over lambda and the bra, under (ucm, ucv); the body is a
// template parameter so that no per-pair switch is if-converted.
template <class T, int BODY, bool EMU>
__device__ __forceinline__ void sweep_pairs(cplx_t<T> *lam, cplx_t<T> *bra, int E, const SweepOp &o, const T *m) {
    using C = cplx_t<T>;
    const uint32_t holes = o.ucm | (1u << o.ut);
    const int nfree = E >> __popc(holes);
    PairWalk w(holes, threadIdx.x, kSweepThreads);
    for (int f = threadIdx.x; f < nfree; f += kSweepThreads) {
        const int e0 = int(w.x | o.ucv), e1 = e0 | (1 << o.ut);
        w.step();
        C l0 = lam[e0], l1 = lam[e1], b0 = bra[e0], b1 = bra[e1];
        body1_sel<T, BODY, EMU>(m, o.uk, l0, l1);
        body1_sel<T, BODY, EMU>(m, o.uk, b0, b1);
        lam[e0] = l0;
        lam[e1] = l1;
        bra[e0] = b0;
        bra[e1] = b1;
    }
}

template <class T, bool EMU>
__device__ __forceinline__ void sweep_udag(cplx_t<T> *lam, cplx_t<T> *bra, int E, const SweepOp &o) {
    using C = cplx_t<T>;
    const T *m = op_u<T>(o);
    if (o.ukind == U_ONE) {
        switch (o.ubody) {
        case B_DIAG: sweep_pairs<T, B_DIAG, EMU>(lam, bra, E, o, m); break;
        case B_PERM: sweep_pairs<T, B_PERM, EMU>(lam, bra, E, o, m); break;
        case B_ANTIDIAG: sweep_pairs<T, B_ANTIDIAG, EMU>(lam, bra, E, o, m); break;
        case B_REAL: sweep_pairs<T, B_REAL, EMU>(lam, bra, E, o, m); break;
        case B_RXLIKE: sweep_pairs<T, B_RXLIKE, EMU>(lam, bra, E, o, m); break;
        default: sweep_pairs<T, B_DENSE, EMU>(lam, bra, E, o, m); break;
        }
    } else if (o.ukind == U_DENSE4) {
        const int qa = o.ut, qb = o.uq2;
        const uint32_t holes = (1u << qa) | (1u << qb);
        const int nfree = E >> 2;
        PairWalk w(holes, threadIdx.x, kSweepThreads);
        for (int f = threadIdx.x; f < nfree; f += kSweepThreads) {
            const int e = int(w.x);
            w.step();
            const int idx[4] = {e, e | (1 << qb), e | (1 << qa), e | (1 << qa) | (1 << qb)};
#pragma unroll
            for (int s = 0; s < 2; s++) {
                C *v = s ? bra : lam;
                C a[4];
#pragma unroll
                for (int c = 0; c < 4; c++) a[c] = v[idx[c]];
#pragma unroll
                for (int r = 0; r < 4; r++) {
                    T xr = 0, xi = 0;
#pragma unroll
                    for (int c = 0; c < 4; c++) {
                        const T mr = m[2 * (r * 4 + c)], mi = m[2 * (r * 4 + c) + 1];
                        xr = fmaT(mr, a[c].x, fmaT(-mi, a[c].y, xr));
                        xi = fmaT(mr, a[c].y, fmaT(mi, a[c].x, xi));
                    }
                    v[idx[r]] = mk<T>(xr, xi);
                }
            }
        }
    }
}

// Im <bra| G |lam> over one generator kind (compile time), under (gcm, gcv).
template <class T, int GKIND>
__device__ __forceinline__ double sweep_gen1(const cplx_t<T> *lam, const cplx_t<T> *bra, int E, const SweepOp &o,
                                             const T *g) {
    using C = cplx_t<T>;
    double acc = 0.0;
    const uint32_t holes = o.gcm | (1u << o.gt);
    const int nfree = E >> __popc(holes);
    PairWalk w(holes, threadIdx.x, kSweepThreads);
    for (int f = threadIdx.x; f < nfree; f += kSweepThreads) {
        const int e0 = int(w.x | o.gcv), e1 = e0 | (1 << o.gt);
        w.step();
        const C k0 = lam[e0], k1 = lam[e1], b0 = bra[e0], b1 = bra[e1];
        T v;
        if constexpr (GKIND == G_Z) {
            v = (b0.x * k0.y - b0.y * k0.x) - (b1.x * k1.y - b1.y * k1.x);
        } else if constexpr (GKIND == G_X) {
            v = (b0.x * k1.y - b0.y * k1.x) + (b1.x * k0.y - b1.y * k0.x);
        } else if constexpr (GKIND == G_Y) {
            v = (b1.x * k0.x + b1.y * k0.y) - (b0.x * k1.x + b0.y * k1.y);
        } else if constexpr (GKIND == G_P1) {
            v = b1.x * k1.y - b1.y * k1.x;
        } else {
            const T y0r = g[0] * k0.x - g[1] * k0.y + g[2] * k1.x - g[3] * k1.y;
            const T y0i = g[0] * k0.y + g[1] * k0.x + g[2] * k1.y + g[3] * k1.x;
            const T y1r = g[4] * k0.x - g[5] * k0.y + g[6] * k1.x - g[7] * k1.y;
            const T y1i = g[4] * k0.y + g[5] * k0.x + g[6] * k1.y + g[7] * k1.x;
            v = (b0.x * y0i - b0.y * y0r) + (b1.x * y1i - b1.y * y1r);
        }
        acc += double(v);
    }
    return acc;
}

// Im <bra| G |lam>, this thread's share (summed over the CTA by the caller).
template <class T>
__device__ __forceinline__ double sweep_gen(const cplx_t<T> *lam, const cplx_t<T> *bra, int E, const SweepOp &o) {
    using C = cplx_t<T>;
    const T *g = op_g<T>(o);
    double acc = 0.0;
    if (o.gkind == G_DENSE4) {
        const int qa = o.gt, qb = o.gq2;
        const uint32_t holes = (1u << qa) | (1u << qb);
        PairWalk w(holes, threadIdx.x, kSweepThreads);
        for (int f = threadIdx.x; f < (E >> 2); f += kSweepThreads) {
            const int e = int(w.x);
            w.step();
            const int idx[4] = {e, e | (1 << qb), e | (1 << qa), e | (1 << qa) | (1 << qb)};
            C a[4];
#pragma unroll
            for (int c = 0; c < 4; c++) a[c] = lam[idx[c]];
#pragma unroll
            for (int r = 0; r < 4; r++) {
                T yr = 0, yi = 0;
#pragma unroll
                for (int c = 0; c < 4; c++) {
                    const T mr = g[2 * (r * 4 + c)], mi = g[2 * (r * 4 + c) + 1];
                    yr = fmaT(mr, a[c].x, fmaT(-mi, a[c].y, yr));
                    yi = fmaT(mr, a[c].y, fmaT(mi, a[c].x, yi));
                }
                const C b = bra[idx[r]];
                acc += double(b.x * yi - b.y * yr);
            }
        }
        return acc;
    }
    switch (o.gkind) {
    case G_Z: return sweep_gen1<T, G_Z>(lam, bra, E, o, g);
    case G_X: return sweep_gen1<T, G_X>(lam, bra, E, o, g);
    case G_Y: return sweep_gen1<T, G_Y>(lam, bra, E, o, g);
    case G_P1: return sweep_gen1<T, G_P1>(lam, bra, E, o, g);
    default: return sweep_gen1<T, G_DENSE>(lam, bra, E, o, g);
    }
}

template <class T, bool EMU>
__global__ void __launch_bounds__(kSweepThreads, 1)
    adjoint_sweep_kernel(const cplx_t<T> *__restrict__ ket, cplx_t<T> *const *__restrict__ bras, int n,
                         const SweepOp *__restrict__ ops, int nops, double *__restrict__ jac, int K) {
    using C = cplx_t<T>;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ double2 red[kSweepThreads / 32];
    const int E = 1 << n;
    C *lam = reinterpret_cast<C *>(smem_raw);
    C *bra = lam + E;
    const int k = blockIdx.x;
    const C *src = bras[k];
    for (int e = threadIdx.x; e < E; e += kSweepThreads) {
        lam[e] = ket[e];
        bra[e] = src[e];
    }
    __syncthreads();
    for (int i = 0; i < nops; i++) {
        const SweepOp &o = ops[i];
        if (o.col >= 0 && o.gkind != G_NONE) {
            const double part = sweep_gen<T>(lam, bra, E, o);
            const double2 s = block_reduce_d2<kSweepThreads>(make_double2(part, 0.0), red);
            if (threadIdx.x == 0) jac[size_t(o.col) * K + k] = s.x;
            __syncthreads();
        }
        sweep_udag<T, EMU>(lam, bra, E, o);
        __syncthreads();
    }
}

// Host: classify one operation of the sweep.
static lgpu_status_t sweep_op_of(const lgpu_adj_op_t &a, uint32_t n, SweepOp *o) {
    *o = SweepOp{};
    auto bit_ok = [&](int b) { return b >= 0 && uint32_t(b) < n; };
    o->col = a.col;
    // U^dag
    if (a.nu == 1) {
        if (!bit_ok(a.ubits[0])) return fail(LGPU_ERR_INVALID_ARG, "adjoint sweep: U bit out of range");
        o->ukind = U_ONE;
        o->ut = a.ubits[0];
        o->ubody = body_of_2x2_host(a.u, o->uk);
        for (int e = 0; e < 8; e++) o->u[e] = a.u[e];
    } else if (a.nu == 2) {
        if (!bit_ok(a.ubits[0]) || !bit_ok(a.ubits[1]) || a.ubits[0] == a.ubits[1])
            return fail(LGPU_ERR_INVALID_ARG, "adjoint sweep: U bits out of range or repeated");
        // controlled form [[I, 0], [0, V]] with the control on the most significant matrix bit
        auto el = [&](int r, int c, int part) { return a.u[2 * (r * 4 + c) + part]; };
        bool ctrl = true;
        for (int r = 0; r < 4; r++)
            for (int c = 0; c < 4; c++) {
                if (r >= 2 && c >= 2) continue;
                const double want = (r == c) ? 1.0 : 0.0;
                if (el(r, c, 0) != want || el(r, c, 1) != 0.0) ctrl = false;
            }
        if (ctrl) {
            double v[8] = {el(2, 2, 0), el(2, 2, 1), el(2, 3, 0), el(2, 3, 1),
                           el(3, 2, 0), el(3, 2, 1), el(3, 3, 0), el(3, 3, 1)};
            o->ukind = U_ONE;
            o->ut = a.ubits[1];
            o->ucm = o->ucv = 1u << a.ubits[0];
            o->ubody = body_of_2x2_host(v, o->uk);
            for (int e = 0; e < 8; e++) o->u[e] = v[e];
        } else {
            o->ukind = U_DENSE4;
            o->ut = a.ubits[0];
            o->uq2 = a.ubits[1];
            for (int e = 0; e < 32; e++) o->u[e] = a.u[e];
        }
    } else {
        return fail(LGPU_ERR_INVALID_ARG, "adjoint sweep: U^dag on 1 or 2 bits");
    }
    // generator
    if (a.ng == 1) {
        if (!bit_ok(a.gbits[0])) return fail(LGPU_ERR_INVALID_ARG, "adjoint sweep: G bit out of range");
        o->gkind = gen_kind(a.g);
        o->gt = a.gbits[0];
        for (int e = 0; e < 8; e++) o->g[e] = a.g[e];
    } else if (a.ng == 2) {
        if (!bit_ok(a.gbits[0]) || !bit_ok(a.gbits[1]) || a.gbits[0] == a.gbits[1])
            return fail(LGPU_ERR_INVALID_ARG, "adjoint sweep: G bits out of range or repeated");
        // |1><1| (x) P on (gbits[0], gbits[1]): P with a control on gbits[0]
        auto el = [&](int r, int c, int part) { return a.g[2 * (r * 4 + c) + part]; };
        bool ctrl = true;
        for (int r = 0; r < 4; r++)
            for (int c = 0; c < 4; c++) {
                if (r >= 2 && c >= 2) continue;
                if (el(r, c, 0) != 0.0 || el(r, c, 1) != 0.0) ctrl = false;
            }
        if (ctrl) {
            double v[8] = {el(2, 2, 0), el(2, 2, 1), el(2, 3, 0), el(2, 3, 1),
                           el(3, 2, 0), el(3, 2, 1), el(3, 3, 0), el(3, 3, 1)};
            o->gkind = gen_kind(v);
            o->gt = a.gbits[1];
            o->gcm = o->gcv = 1u << a.gbits[0];
            for (int e = 0; e < 8; e++) o->g[e] = v[e];
        } else {
            o->gkind = G_DENSE4;
            o->gt = a.gbits[0];
            o->gq2 = a.gbits[1];
            for (int e = 0; e < 32; e++) o->g[e] = a.g[e];
        }
    } else if (a.ng == 0) {
        o->gkind = G_NONE;
        o->col = -1;
    } else {
        return fail(LGPU_ERR_INVALID_ARG, "adjoint sweep: generator on 0, 1 or 2 bits");
    }
    if (a.ng > 0 && a.col < 0) return fail(LGPU_ERR_INVALID_ARG, "adjoint sweep: negative Jacobian column");
    for (int e = 0; e < 32; e++) {
        o->uf[e] = float(o->u[e]);
        o->gf[e] = float(o->g[e]);
    }
    return LGPU_OK;
}

template <class T, bool EMU>
static lgpu_status_t sweep_launch(const void *ket, void *const *dbras, uint32_t nbras, uint32_t n, const SweepOp *dops,
                                  uint32_t nops, double *jac, cudaStream_t s) {
    const size_t smem = 2 * (size_t(1) << n) * sizeof(cplx_t<T>);
    static std::atomic<size_t> attr[64];
    LGPU_TRY(ensure_smem(reinterpret_cast<const void *>(adjoint_sweep_kernel<T, EMU>), smem, attr));
    adjoint_sweep_kernel<T, EMU><<<nbras, kSweepThreads, smem, s>>>(
        static_cast<const cplx_t<T> *>(ket), reinterpret_cast<cplx_t<T> *const *>(dbras), int(n), dops, int(nops), jac,
        int(nbras));
    LGPU_CHECK_LAUNCH();
    return LGPU_OK;
}

// ---------------------------------------------------------------------------
// Fused adjoint blocks (complex128): several operations of the reverse sweep
// per pass.  Each CTA loads a tile of lambda and of each bra (the tile bits =
// the low run 0..m-1 plus up to 6 high bits, as the fused gate blocks),
// converts them in place to float-float (lgpu_df64.cuh) and runs the steps in
// order; a step reads a pair, adds Im <bra| G |lambda> to the thread's
// float-float sum and applies U^dag to lambda and the bras.  The sums are
// reduced per warp (shuffles), kept per warp in shared memory across the
// CTA's tiles, written per CTA and summed over CTAs in a fixed order.
// ---------------------------------------------------------------------------
constexpr int kAdjBlockSteps = 48;
constexpr int kAdjBlockBras = 2;
constexpr int kAdjBlockThreads = 256;

constexpr int kAdjGroupBits = 4;   // phase group: table over at most 4 tile positions
constexpr int kAdjGroupGrads = 4;  // and at most 4 gradient steps
constexpr uint8_t kAdjPhaseGroup = 2;

struct AStep {
    uint8_t q;      // tile position of the target
    uint8_t body;   // Body1 of U^dag
    int8_t gk;      // GenKind, G_NONE: no gradient
    uint8_t pad;    // 1: U^dag = diag(+-1, +-1), sign flips; kAdjPhaseGroup: a phase group
    int32_t slot;   // accumulator slot of a gradient step (phase group: its table in gtab)
    uint32_t in_mask, in_val;    // controls inside the tile (phase group: the table positions)
    uint64_t out_mask, out_val;  // controls outside the tile (state bits)
    DF u[8];
    DF g[8];
    // phase group: its gradient steps (tile position, G_Z or G_P1, slot)
    uint8_t ng;
    uint8_t gq[kAdjGroupGrads];
    int8_t gkd[kAdjGroupGrads];
    int16_t gslot[kAdjGroupGrads];
};

template <class I> struct AdjBlockParams {
    Holes holes;
    I ntiles;
    int k, m;
    int nsteps, nslots, nb;
    I hi_off[64];
    double2 *ket;
    double2 *bras[kAdjBlockBras];
    double *partials;  // [gridDim.x][nslots][nb]
    int in_ff, out_ff;  // complex128: the states are read / left in float-float form
    AStep steps[kAdjBlockSteps];
    // phase-group tables (a group step's slot indexes them): entries (re.hi, re.lo, im.hi, im.lo)
    float4 gtab[kAdjBlockSteps / 2][1 << kAdjGroupBits];
};
static_assert(sizeof(AdjBlockParams<uint64_t>) <= 32000, "adjoint block parameters exceed the 32 KB limit");

__device__ __forceinline__ void adj_cp_async16(void *smem_dst, const void *gsrc) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(static_cast<uint32_t>(__cvta_generic_to_shared(smem_dst))),
                 "l"(gsrc)
                 : "memory");
}

// Im(conj(b) G k) over the pair, G by kind.
template <int GK>
__device__ __forceinline__ DF gexp_df(const DF *g, const DF (&b)[4], const DF (&k)[4]) {
    // b = (b0r, b0i, b1r, b1i), k likewise
    if constexpr (GK == G_Z)
        return df_sum<4>({df_mul(b[0], k[1]), df_neg(df_mul(b[1], k[0])), df_neg(df_mul(b[2], k[3])), df_mul(b[3], k[2])});
    else if constexpr (GK == G_X)
        return df_sum<4>({df_mul(b[0], k[3]), df_neg(df_mul(b[1], k[2])), df_mul(b[2], k[1]), df_neg(df_mul(b[3], k[0]))});
    else if constexpr (GK == G_Y)
        return df_sum<4>({df_mul(b[2], k[0]), df_mul(b[3], k[1]), df_neg(df_mul(b[0], k[2])), df_neg(df_mul(b[1], k[3]))});
    else if constexpr (GK == G_P1)
        return df_sum<2>({df_mul(b[2], k[3]), df_neg(df_mul(b[3], k[2]))});
    else {
        // y = G k, then Im(conj(b0) y0 + conj(b1) y1)
        const DF y0r = df_sum<4>({df_mul(g[0], k[0]), df_neg(df_mul(g[1], k[1])), df_mul(g[2], k[2]), df_neg(df_mul(g[3], k[3]))});
        const DF y0i = df_sum<4>({df_mul(g[0], k[1]), df_mul(g[1], k[0]), df_mul(g[2], k[3]), df_mul(g[3], k[2])});
        const DF y1r = df_sum<4>({df_mul(g[4], k[0]), df_neg(df_mul(g[5], k[1])), df_mul(g[6], k[2]), df_neg(df_mul(g[7], k[3]))});
        const DF y1i = df_sum<4>({df_mul(g[4], k[1]), df_mul(g[5], k[0]), df_mul(g[6], k[3]), df_mul(g[7], k[2])});
        return df_sum<4>({df_mul(b[0], y0i), df_neg(df_mul(b[1], y0r)), df_mul(b[2], y1i), df_neg(df_mul(b[3], y1r))});
    }
}

__device__ __forceinline__ DF df_shfl_xor(DF v, int o) {
    return DF{__shfl_xor_sync(0xffffffffu, v.hi, o), __shfl_xor_sync(0xffffffffu, v.lo, o)};
}

// One step on the tile: the pairs (e0, e0 | 1 << q) with the in-tile controls
// set.  BODY / GK at compile time (G_NONE: U^dag only).  Amplitudes are float4
// (re.hi, im.hi, re.lo, im.lo); U^dag runs as paired float-float lanes
// (re, im) (lgpu_df2.cuh), the overlap in scalar float-float.
template <int BODY>
__device__ __forceinline__ void adj_udag_pair(const DF2 (&c)[8], float s0, float s1, float4 &a, float4 &b) {
    if constexpr (BODY == kDfSignDiag) {  // diag(+-1, +-1): exact sign flips
        a = make_float4(a.x * s0, a.y * s0, a.z * s0, a.w * s0);
        b = make_float4(b.x * s1, b.y * s1, b.z * s1, b.w * s1);
    } else if constexpr (BODY == B_PERM) {
        const float4 t = a;
        a = b;
        b = t;
    } else {
        DF2 x{f2_pack(a.x, a.y), f2_pack(a.z, a.w)}, y{f2_pack(b.x, b.y), f2_pack(b.z, b.w)};
        body1_df2<BODY>(c, x, y);
        a = make_float4(f2_x(x.hi), f2_y(x.hi), f2_x(x.lo), f2_y(x.lo));
        b = make_float4(f2_x(y.hi), f2_y(y.hi), f2_x(y.lo), f2_y(y.lo));
    }
}

template <int BODY, int GK, int NB>
__device__ __forceinline__ void adj_block_step(float4 *kt, float4 *const (&bt)[kAdjBlockBras], int E, const AStep &st,
                                               DF (&acc)[kAdjBlockBras]) {
    DF u[8], g[8];
#pragma unroll
    for (int i = 0; i < 8; i++) u[i] = st.u[i];
    if constexpr (GK == G_DENSE) {
#pragma unroll
        for (int i = 0; i < 8; i++) g[i] = st.g[i];
    }
    DF2 c[8];
    if constexpr (BODY != kDfSignDiag && BODY != B_PERM) df2_coeffs(u, c);
    const float s0 = u[0].hi, s1 = u[6].hi;
    const uint32_t holes = st.in_mask | (1u << st.q);
    const int nfree = E >> __popc(holes);
    PairWalk w(holes, threadIdx.x, kAdjBlockThreads);
    for (int f = threadIdx.x; f < nfree; f += kAdjBlockThreads) {
        const int e0 = int(w.x | st.in_val);
        const int e1 = e0 | (1 << st.q);
        w.step();
        const int s0i = swz<double>(e0), s1i = swz<double>(e1);
        float4 ka = kt[s0i], kb = kt[s1i];
        const DF kv[4] = {DF{ka.x, ka.z}, DF{ka.y, ka.w}, DF{kb.x, kb.z}, DF{kb.y, kb.w}};
#pragma unroll
        for (int b = 0; b < NB; b++) {
            float4 ba = bt[b][s0i], bb = bt[b][s1i];
            if constexpr (GK != G_NONE) {
                const DF bv[4] = {DF{ba.x, ba.z}, DF{ba.y, ba.w}, DF{bb.x, bb.z}, DF{bb.y, bb.w}};
                acc[b] = df_sum<2>({acc[b], gexp_df<GK>(g, bv, kv)});
            }
            adj_udag_pair<BODY>(c, s0, s1, ba, bb);
            bt[b][s0i] = ba;
            bt[b][s1i] = bb;
        }
        adj_udag_pair<BODY>(c, s0, s1, ka, kb);
        kt[s0i] = ka;
        kt[s1i] = kb;
    }
}

// A phase group (host: consecutive uncontrolled diagonal steps, RZ,
// PhaseShift or gradient-free, on at most kAdjGroupBits tile positions).
// Their U^dag are diagonal and commute with each other and with the
// generators Z and P1, so every overlap Im <bra| G_j |lambda> equals its value
// before any of the group's U^dag is applied: one product Im(conj(bra)
// lambda) per amplitude serves all of them (G_Z: + for target bit 0, - for 1;
// G_P1: bit 1 only), and one table of the U^dag products (staged in shared
// memory by the caller, entries (re.hi, re.lo, im.hi, im.lo)) multiplies
// lambda and the bras.
template <int NB>
__device__ __forceinline__ void adj_phase_group(float4 *kt, float4 *const (&bt)[kAdjBlockBras], int E, const AStep &st,
                                                const float4 *tab, DF (&acc)[kAdjGroupGrads][kAdjBlockBras]) {
    int sh[kAdjGroupBits];  // index bit b = tile bit q_b (ascending): (e >> (q_b - b)) & (1 << b)
    {
        uint32_t mm = st.in_mask;
#pragma unroll
        for (int b = 0; b < kAdjGroupBits; b++) {
            sh[b] = mm ? (__ffs(int(mm)) - 1 - b) : (31 - b);
            mm &= mm - 1u;
        }
    }
    const int ng = st.ng;
    for (int e = threadIdx.x; e < E; e += kAdjBlockThreads) {
        int idx = 0;
#pragma unroll
        for (int b = 0; b < kAdjGroupBits; b++) idx |= (e >> sh[b]) & (1 << b);
        const float4 t = tab[idx];
        const DF2 c1{f2_pack(t.x, t.x), f2_pack(t.y, t.y)}, c2{f2_pack(-t.z, t.z), f2_pack(-t.w, t.w)};
        auto phase = [&](float4 &a) {
            const DF2 x{f2_pack(a.x, a.y), f2_pack(a.z, a.w)}, xs{f2_pack(a.y, a.x), f2_pack(a.w, a.z)};
            const DF2 y = df2_sum<2>({df2_mul(c1, x), df2_mul(c2, xs)});
            a = make_float4(f2_x(y.hi), f2_y(y.hi), f2_x(y.lo), f2_y(y.lo));
        };
        const int si = swz<double>(e);
        float4 kv = kt[si];
        const DF kr{kv.x, kv.z}, ki{kv.y, kv.w};
#pragma unroll
        for (int b = 0; b < NB; b++) {
            float4 bv = bt[b][si];
            if (ng > 0) {
                const DF pr = df_sum<2>({df_mul(DF{bv.x, bv.z}, ki), df_neg(df_mul(DF{bv.y, bv.w}, kr))});
#pragma unroll
                for (int j = 0; j < kAdjGroupGrads; j++) {
                    if (j >= ng) break;
                    const int bit = (e >> st.gq[j]) & 1;
                    const DF c = st.gkd[j] == G_Z ? (bit ? df_neg(pr) : pr) : (bit ? pr : DF{0.0f, 0.0f});
                    acc[j][b] = df_sum<2>({acc[j][b], c});
                }
            }
            phase(bv);
            bt[b][si] = bv;
        }
        phase(kv);
        kt[si] = kv;
    }
}

template <int NB>
__device__ __forceinline__ void adj_block_dispatch(float4 *kt, float4 *const (&bt)[kAdjBlockBras], int E,
                                                   const AStep &st, DF (&acc)[kAdjBlockBras]) {
    switch (st.gk) {
    case G_NONE:
        switch (st.pad == 1 ? kDfSignDiag : int(st.body)) {
        case kDfSignDiag: adj_block_step<kDfSignDiag, G_NONE, NB>(kt, bt, E, st, acc); break;
        case B_DIAG: adj_block_step<B_DIAG, G_NONE, NB>(kt, bt, E, st, acc); break;
        case B_PERM: adj_block_step<B_PERM, G_NONE, NB>(kt, bt, E, st, acc); break;
        case B_ANTIDIAG: adj_block_step<B_ANTIDIAG, G_NONE, NB>(kt, bt, E, st, acc); break;
        case B_REAL: adj_block_step<B_REAL, G_NONE, NB>(kt, bt, E, st, acc); break;
        case B_RXLIKE: adj_block_step<B_RXLIKE, G_NONE, NB>(kt, bt, E, st, acc); break;
        default: adj_block_step<B_DENSE, G_NONE, NB>(kt, bt, E, st, acc); break;
        }
        break;
    case G_X:  // RX-like rotations
        if (st.body == B_RXLIKE) adj_block_step<B_RXLIKE, G_X, NB>(kt, bt, E, st, acc);
        else adj_block_step<B_DENSE, G_X, NB>(kt, bt, E, st, acc);
        break;
    case G_Y:  // RY: real rotation
        if (st.body == B_REAL) adj_block_step<B_REAL, G_Y, NB>(kt, bt, E, st, acc);
        else adj_block_step<B_DENSE, G_Y, NB>(kt, bt, E, st, acc);
        break;
    case G_Z:  // RZ: diagonal
        if (st.body == B_DIAG) adj_block_step<B_DIAG, G_Z, NB>(kt, bt, E, st, acc);
        else adj_block_step<B_DENSE, G_Z, NB>(kt, bt, E, st, acc);
        break;
    case G_P1:  // PhaseShift: diagonal
        if (st.body == B_DIAG) adj_block_step<B_DIAG, G_P1, NB>(kt, bt, E, st, acc);
        else adj_block_step<B_DENSE, G_P1, NB>(kt, bt, E, st, acc);
        break;
    default: adj_block_step<B_DENSE, G_DENSE, NB>(kt, bt, E, st, acc); break;
    }
}

template <class I, int NB>
__global__ void __launch_bounds__(kAdjBlockThreads, 3) adjoint_block_kernel(const AdjBlockParams<I> p) {
    extern __shared__ __align__(128) unsigned char adj_smem[];
    const int E = 1 << p.k;
    float4 *kt = reinterpret_cast<float4 *>(adj_smem);
    float4 *bt[kAdjBlockBras];
#pragma unroll
    for (int b = 0; b < kAdjBlockBras; b++) bt[b] = kt + size_t(b + 1) * E;
    constexpr int W = kAdjBlockThreads / 32;
    DF *wacc = reinterpret_cast<DF *>(kt + size_t(NB + 1) * E);  // [nslots][NB][W]
    for (int i = threadIdx.x; i < p.nslots * NB * W; i += kAdjBlockThreads) wacc[i] = DF{0.0f, 0.0f};
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int lowmask = (1 << p.m) - 1;
    __syncthreads();
    for (I tau = blockIdx.x; tau < p.ntiles; tau += I(gridDim.x)) {
        const I base = insert_holes<I>(tau, p.holes);
        for (int e = threadIdx.x; e < E; e += kAdjBlockThreads) {
            const I gi = base + p.hi_off[e >> p.m] + I(e & lowmask);
            adj_cp_async16(&kt[swz<double>(e)], &p.ket[gi]);
#pragma unroll
            for (int b = 0; b < NB; b++) adj_cp_async16(&bt[b][swz<double>(e)], &p.bras[b][gi]);
        }
        asm volatile("cp.async.commit_group;" ::: "memory");
        asm volatile("cp.async.wait_group 0;" ::: "memory");
        __syncthreads();
        if (!p.in_ff) {  // complex128 -> float-float in place (same 16 bytes per amplitude)
            for (int e = threadIdx.x; e < E * (NB + 1); e += kAdjBlockThreads) {
                const double2 v = reinterpret_cast<const double2 *>(kt)[e];
                const DF r = df_from_double(v.x), i = df_from_double(v.y);
                kt[e] = make_float4(r.hi, i.hi, r.lo, i.lo);
            }
            __syncthreads();
        }
        for (int si = 0; si < p.nsteps; si++) {
            const AStep &st = p.steps[si];
            if ((uint64_t(base) & st.out_mask) != st.out_val) continue;  // tile-uniform
            if (st.pad == kAdjPhaseGroup) {
                float4 *tab = reinterpret_cast<float4 *>(wacc + size_t(p.nslots) * NB * W);
                if (threadIdx.x < (1 << kAdjGroupBits))
                    tab[threadIdx.x] = p.gtab[st.slot][threadIdx.x];
                __syncthreads();
                DF gacc[kAdjGroupGrads][kAdjBlockBras];
#pragma unroll
                for (int j = 0; j < kAdjGroupGrads; j++)
#pragma unroll
                    for (int b = 0; b < kAdjBlockBras; b++) gacc[j][b] = DF{0.0f, 0.0f};
                adj_phase_group<NB>(kt, bt, E, st, tab, gacc);
#pragma unroll
                for (int j = 0; j < kAdjGroupGrads; j++) {
                    if (j >= st.ng) break;
#pragma unroll
                    for (int b = 0; b < NB; b++) {
                        DF v = gacc[j][b];
#pragma unroll
                        for (int o = 16; o > 0; o >>= 1) v = df_sum<2>({v, df_shfl_xor(v, o)});
                        if (lane == 0) {
                            DF &slot = wacc[(st.gslot[j] * NB + b) * W + warp];
                            slot = df_sum<2>({slot, v});
                        }
                    }
                }
                __syncthreads();
                continue;
            }
            DF acc[kAdjBlockBras];
#pragma unroll
            for (int b = 0; b < kAdjBlockBras; b++) acc[b] = DF{0.0f, 0.0f};
            adj_block_dispatch<NB>(kt, bt, E, st, acc);
            if (st.gk != G_NONE) {
#pragma unroll
                for (int b = 0; b < NB; b++) {
                    DF v = acc[b];
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1) v = df_sum<2>({v, df_shfl_xor(v, o)});
                    if (lane == 0) {
                        DF &slot = wacc[(st.slot * NB + b) * W + warp];
                        slot = df_sum<2>({slot, v});
                    }
                }
            }
            __syncthreads();
        }
        // streamed out: float-float as it is, or converted to complex128
        for (int e = threadIdx.x; e < E; e += kAdjBlockThreads) {
            const I gi = base + p.hi_off[e >> p.m] + I(e & lowmask);
            const float4 v = kt[swz<double>(e)];
            if (p.out_ff) {
                __stcs(reinterpret_cast<float4 *>(&p.ket[gi]), v);
#pragma unroll
                for (int b = 0; b < NB; b++) __stcs(reinterpret_cast<float4 *>(&p.bras[b][gi]), bt[b][swz<double>(e)]);
            } else {
                __stcs(&p.ket[gi], make_double2(df_to_double(DF{v.x, v.z}), df_to_double(DF{v.y, v.w})));
#pragma unroll
                for (int b = 0; b < NB; b++) {
                    const float4 x = bt[b][swz<double>(e)];
                    __stcs(&p.bras[b][gi], make_double2(df_to_double(DF{x.x, x.z}), df_to_double(DF{x.y, x.w})));
                }
            }
        }
        __syncthreads();
    }
    // per CTA: the warps' sums in warp order
    for (int i = threadIdx.x; i < p.nslots * NB; i += kAdjBlockThreads) {
        DF t = wacc[i * W];
        for (int w = 1; w < W; w++) t = df_sum<2>({t, wacc[i * W + w]});
        p.partials[size_t(blockIdx.x) * p.nslots * NB + i] = df_to_double(t);
    }
}

// The same blocks for complex64: float2 tiles, FP32 bodies and overlaps
// (float sums per step and thread, double per-warp slots).
template <int GK>
__device__ __forceinline__ float gexp_f32(const float *g, float2 b0, float2 b1, float2 k0, float2 k1) {
    if constexpr (GK == G_Z) return (b0.x * k0.y - b0.y * k0.x) - (b1.x * k1.y - b1.y * k1.x);
    else if constexpr (GK == G_X) return (b0.x * k1.y - b0.y * k1.x) + (b1.x * k0.y - b1.y * k0.x);
    else if constexpr (GK == G_Y) return (b1.x * k0.x + b1.y * k0.y) - (b0.x * k1.x + b0.y * k1.y);
    else if constexpr (GK == G_P1) return b1.x * k1.y - b1.y * k1.x;
    else {
        const float y0r = g[0] * k0.x - g[1] * k0.y + g[2] * k1.x - g[3] * k1.y;
        const float y0i = g[0] * k0.y + g[1] * k0.x + g[2] * k1.y + g[3] * k1.x;
        const float y1r = g[4] * k0.x - g[5] * k0.y + g[6] * k1.x - g[7] * k1.y;
        const float y1i = g[4] * k0.y + g[5] * k0.x + g[6] * k1.y + g[7] * k1.x;
        return (b0.x * y0i - b0.y * y0r) + (b1.x * y1i - b1.y * y1r);
    }
}

template <int BODY, int GK, int NB>
__device__ __forceinline__ void adj_block_step_f32(float2 *kt, float2 *const (&bt)[kAdjBlockBras], int E,
                                                   const AStep &st, float (&acc)[kAdjBlockBras]) {
    float u[8], g[8];
#pragma unroll
    for (int i = 0; i < 8; i++) {
        u[i] = st.u[i].hi;
        g[i] = st.g[i].hi;
    }
    const uint32_t holes = st.in_mask | (1u << st.q);
    const int nfree = E >> __popc(holes);
    PairWalk w(holes, threadIdx.x, kAdjBlockThreads);
    for (int f = threadIdx.x; f < nfree; f += kAdjBlockThreads) {
        const int e0 = int(w.x | st.in_val);
        const int e1 = e0 | (1 << st.q);
        w.step();
        const int s0 = swz<float>(e0), s1 = swz<float>(e1);
        float2 k0 = kt[s0], k1 = kt[s1];
#pragma unroll
        for (int b = 0; b < NB; b++) {
            float2 b0 = bt[b][s0], b1 = bt[b][s1];
            if constexpr (GK != G_NONE) acc[b] += gexp_f32<GK>(g, b0, b1, k0, k1);
            body1<float, BODY>(u, b0, b1);
            bt[b][s0] = b0;
            bt[b][s1] = b1;
        }
        body1<float, BODY>(u, k0, k1);
        kt[s0] = k0;
        kt[s1] = k1;
    }
}

// A phase group on complex64 tiles (see adj_phase_group): FP32 products,
// the table entries as float2 (staged in shared memory by the caller).
template <int NB>
__device__ __forceinline__ void adj_phase_group_f32(float2 *kt, float2 *const (&bt)[kAdjBlockBras], int E,
                                                    const AStep &st, const float2 *tab,
                                                    float (&acc)[kAdjGroupGrads][kAdjBlockBras]) {
    int sh[kAdjGroupBits];
    {
        uint32_t mm = st.in_mask;
#pragma unroll
        for (int b = 0; b < kAdjGroupBits; b++) {
            sh[b] = mm ? (__ffs(int(mm)) - 1 - b) : (31 - b);
            mm &= mm - 1u;
        }
    }
    const int ng = st.ng;
    for (int e = threadIdx.x; e < E; e += kAdjBlockThreads) {
        int idx = 0;
#pragma unroll
        for (int b = 0; b < kAdjGroupBits; b++) idx |= (e >> sh[b]) & (1 << b);
        const float2 t = tab[idx];
        const int si = swz<float>(e);
        float2 kv = kt[si];
#pragma unroll
        for (int b = 0; b < NB; b++) {
            float2 bv = bt[b][si];
            if (ng > 0) {
                const float pr = bv.x * kv.y - bv.y * kv.x;
#pragma unroll
                for (int j = 0; j < kAdjGroupGrads; j++) {
                    if (j >= ng) break;
                    const int bit = (e >> st.gq[j]) & 1;
                    acc[j][b] += st.gkd[j] == G_Z ? (bit ? -pr : pr) : (bit ? pr : 0.0f);
                }
            }
            bt[b][si] = make_float2(t.x * bv.x - t.y * bv.y, t.x * bv.y + t.y * bv.x);
        }
        kt[si] = make_float2(t.x * kv.x - t.y * kv.y, t.x * kv.y + t.y * kv.x);
    }
}

template <int NB>
__device__ __forceinline__ void adj_block_dispatch_f32(float2 *kt, float2 *const (&bt)[kAdjBlockBras], int E,
                                                       const AStep &st, float (&acc)[kAdjBlockBras]) {
    switch (st.gk) {
    case G_NONE:
        switch (st.body) {
        case B_DIAG: adj_block_step_f32<B_DIAG, G_NONE, NB>(kt, bt, E, st, acc); break;
        case B_PERM: adj_block_step_f32<B_PERM, G_NONE, NB>(kt, bt, E, st, acc); break;
        case B_ANTIDIAG: adj_block_step_f32<B_ANTIDIAG, G_NONE, NB>(kt, bt, E, st, acc); break;
        case B_REAL: adj_block_step_f32<B_REAL, G_NONE, NB>(kt, bt, E, st, acc); break;
        case B_RXLIKE: adj_block_step_f32<B_RXLIKE, G_NONE, NB>(kt, bt, E, st, acc); break;
        default: adj_block_step_f32<B_DENSE, G_NONE, NB>(kt, bt, E, st, acc); break;
        }
        break;
    case G_X:
        if (st.body == B_RXLIKE) adj_block_step_f32<B_RXLIKE, G_X, NB>(kt, bt, E, st, acc);
        else adj_block_step_f32<B_DENSE, G_X, NB>(kt, bt, E, st, acc);
        break;
    case G_Y:
        if (st.body == B_REAL) adj_block_step_f32<B_REAL, G_Y, NB>(kt, bt, E, st, acc);
        else adj_block_step_f32<B_DENSE, G_Y, NB>(kt, bt, E, st, acc);
        break;
    case G_Z:
        if (st.body == B_DIAG) adj_block_step_f32<B_DIAG, G_Z, NB>(kt, bt, E, st, acc);
        else adj_block_step_f32<B_DENSE, G_Z, NB>(kt, bt, E, st, acc);
        break;
    case G_P1:
        if (st.body == B_DIAG) adj_block_step_f32<B_DIAG, G_P1, NB>(kt, bt, E, st, acc);
        else adj_block_step_f32<B_DENSE, G_P1, NB>(kt, bt, E, st, acc);
        break;
    default: adj_block_step_f32<B_DENSE, G_DENSE, NB>(kt, bt, E, st, acc); break;
    }
}

template <class I, int NB>
__global__ void __launch_bounds__(kAdjBlockThreads, 3) adjoint_block_f32_kernel(const AdjBlockParams<I> p) {
    extern __shared__ __align__(128) unsigned char adj_smem[];
    const int E = 1 << p.k;
    float2 *kt = reinterpret_cast<float2 *>(adj_smem);
    float2 *bt[kAdjBlockBras];
#pragma unroll
    for (int b = 0; b < kAdjBlockBras; b++) bt[b] = kt + size_t(b + 1) * E;
    constexpr int W = kAdjBlockThreads / 32;
    double *wacc = reinterpret_cast<double *>(kt + size_t(NB + 1) * E);  // [nslots][NB][W]
    for (int i = threadIdx.x; i < p.nslots * NB * W; i += kAdjBlockThreads) wacc[i] = 0.0;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int lowmask = (1 << p.m) - 1;
    float2 *ket = reinterpret_cast<float2 *>(p.ket);
    float2 *bras[kAdjBlockBras];
#pragma unroll
    for (int b = 0; b < kAdjBlockBras; b++) bras[b] = reinterpret_cast<float2 *>(p.bras[b]);
    __syncthreads();
    for (I tau = blockIdx.x; tau < p.ntiles; tau += I(gridDim.x)) {
        const I base = insert_holes<I>(tau, p.holes);
        // 16-byte chunks = 2 amplitudes of the low run (m >= 1)
        for (int c = threadIdx.x; c < E / 2; c += kAdjBlockThreads) {
            const int e = 2 * c;
            const I gi = base + p.hi_off[e >> p.m] + I(e & lowmask);
            adj_cp_async16(&kt[swz<float>(e)], &ket[gi]);
#pragma unroll
            for (int b = 0; b < NB; b++) adj_cp_async16(&bt[b][swz<float>(e)], &bras[b][gi]);
        }
        asm volatile("cp.async.commit_group;" ::: "memory");
        asm volatile("cp.async.wait_group 0;" ::: "memory");
        __syncthreads();
        for (int si = 0; si < p.nsteps; si++) {
            const AStep &st = p.steps[si];
            if ((uint64_t(base) & st.out_mask) != st.out_val) continue;  // tile-uniform
            if (st.pad == kAdjPhaseGroup) {
                float2 *tab = reinterpret_cast<float2 *>(wacc + size_t(p.nslots) * NB * W);
                if (threadIdx.x < (1 << kAdjGroupBits))
                    tab[threadIdx.x] = make_float2(p.gtab[st.slot][threadIdx.x].x, p.gtab[st.slot][threadIdx.x].z);
                __syncthreads();
                float gacc[kAdjGroupGrads][kAdjBlockBras];
#pragma unroll
                for (int j = 0; j < kAdjGroupGrads; j++)
#pragma unroll
                    for (int b = 0; b < kAdjBlockBras; b++) gacc[j][b] = 0.0f;
                adj_phase_group_f32<NB>(kt, bt, E, st, tab, gacc);
#pragma unroll
                for (int j = 0; j < kAdjGroupGrads; j++) {
                    if (j >= st.ng) break;
#pragma unroll
                    for (int b = 0; b < NB; b++) {
                        float v = gacc[j][b];
#pragma unroll
                        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
                        if (lane == 0) wacc[(st.gslot[j] * NB + b) * W + warp] += double(v);
                    }
                }
                __syncthreads();
                continue;
            }
            float acc[kAdjBlockBras];
#pragma unroll
            for (int b = 0; b < kAdjBlockBras; b++) acc[b] = 0.0f;
            adj_block_dispatch_f32<NB>(kt, bt, E, st, acc);
            if (st.gk != G_NONE) {
#pragma unroll
                for (int b = 0; b < NB; b++) {
                    float v = acc[b];
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
                    if (lane == 0) wacc[(st.slot * NB + b) * W + warp] += double(v);
                }
            }
            __syncthreads();
        }
        for (int c = threadIdx.x; c < E / 2; c += kAdjBlockThreads) {
            const int e = 2 * c;
            const I gi = base + p.hi_off[e >> p.m] + I(e & lowmask);
            __stcs(reinterpret_cast<float4 *>(&ket[gi]), *reinterpret_cast<const float4 *>(&kt[swz<float>(e)]));
#pragma unroll
            for (int b = 0; b < NB; b++)
                __stcs(reinterpret_cast<float4 *>(&bras[b][gi]), *reinterpret_cast<const float4 *>(&bt[b][swz<float>(e)]));
        }
        __syncthreads();
    }
    for (int i = threadIdx.x; i < p.nslots * NB; i += kAdjBlockThreads) {
        double t = 0.0;
        for (int w = 0; w < W; w++) t += wacc[i * W + w];
        p.partials[size_t(blockIdx.x) * p.nslots * NB + i] = t;
    }
}

// jac[col[s] * stride + b] = sum over CTAs (in CTA order) of the partials.
// One warp per (slot, bra): lane l sums the CTAs l, l + 32, ... in order, then
// a fixed shuffle tree adds the lanes (the same order every run).
__global__ void adjoint_block_reduce(const double *__restrict__ partials, int nctas, int nslots, int nb,
                                     const int *__restrict__ cols, double *__restrict__ jac, int stride) {
    const int i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (i >= nslots * nb) return;  // whole warps leave together
    double t = 0.0;
    for (int c = lane; c < nctas; c += 32) t += partials[size_t(c) * nslots * nb + i];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if (lane == 0) jac[size_t(cols[i / nb]) * stride + (i % nb)] = t;
}

// ---------------------------------------------------------------------------
// The whole small-state sweep in float-float (complex128): lambda and the bra
// are converted once while they are loaded into shared memory, and every
// operation, generator overlap and block sum runs on the float-float copies
// (no FP64 instruction).  Same order, operations and results as
// adjoint_sweep_kernel.
// ---------------------------------------------------------------------------
struct SweepDF {
    DF u[32];
    DF g[32];
    int sign_diag;  // U^dag = diag(+-1, +-1) on one bit
};

template <int BODY, class OP>
__device__ __forceinline__ void sweep_pairs_df(float4 *lam, float4 *bra, int E, const OP &o, const DF *mp) {
    DF m[8];
#pragma unroll
    for (int i = 0; i < 8; i++) m[i] = mp[i];
    const uint32_t holes = o.ucm | (1u << o.ut);
    const int nfree = E >> __popc(holes);
    PairWalk w(holes, threadIdx.x, kSweepThreads);
    for (int f = threadIdx.x; f < nfree; f += kSweepThreads) {
        const int e0 = int(w.x | o.ucv), e1 = e0 | (1 << o.ut);
        w.step();
#pragma unroll
        for (int st = 0; st < 2; st++) {
            float4 *v = st ? bra : lam;
            const float4 a = v[e0], b = v[e1];
            DF xr{a.x, a.y}, xi{a.z, a.w}, yr{b.x, b.y}, yi{b.z, b.w};
            body1_dfv<BODY>(m, xr, xi, yr, yi);
            v[e0] = make_float4(xr.hi, xr.lo, xi.hi, xi.lo);
            v[e1] = make_float4(yr.hi, yr.lo, yi.hi, yi.lo);
        }
    }
}

template <class OP>
__device__ __forceinline__ void sweep_udag_df(float4 *lam, float4 *bra, int E, const OP &o, const SweepDF &d) {
    if (o.ukind == U_ONE) {
        switch (d.sign_diag ? kDfSignDiag : o.ubody) {
        case kDfSignDiag: sweep_pairs_df<kDfSignDiag>(lam, bra, E, o, d.u); break;
        case B_DIAG: sweep_pairs_df<B_DIAG>(lam, bra, E, o, d.u); break;
        case B_PERM: sweep_pairs_df<B_PERM>(lam, bra, E, o, d.u); break;
        case B_ANTIDIAG: sweep_pairs_df<B_ANTIDIAG>(lam, bra, E, o, d.u); break;
        case B_REAL: sweep_pairs_df<B_REAL>(lam, bra, E, o, d.u); break;
        case B_RXLIKE: sweep_pairs_df<B_RXLIKE>(lam, bra, E, o, d.u); break;
        default: sweep_pairs_df<B_DENSE>(lam, bra, E, o, d.u); break;
        }
    } else if (o.ukind == U_DENSE4) {
        const int qa = o.ut, qb = o.uq2;
        const uint32_t holes = (1u << qa) | (1u << qb);
        PairWalk w(holes, threadIdx.x, kSweepThreads);
        for (int f = threadIdx.x; f < (E >> 2); f += kSweepThreads) {
            const int e = int(w.x);
            w.step();
            const int idx[4] = {e, e | (1 << qb), e | (1 << qa), e | (1 << qa) | (1 << qb)};
#pragma unroll
            for (int st = 0; st < 2; st++) {
                float4 *v = st ? bra : lam;
                DF ar[4], ai[4];
#pragma unroll
                for (int c = 0; c < 4; c++) {
                    const float4 x = v[idx[c]];
                    ar[c] = DF{x.x, x.y};
                    ai[c] = DF{x.z, x.w};
                }
#pragma unroll
                for (int r = 0; r < 4; r++) {
                    DF tr[8], ti[8];
#pragma unroll
                    for (int c = 0; c < 4; c++) {
                        const DF mre = d.u[2 * (r * 4 + c)], mim = d.u[2 * (r * 4 + c) + 1];
                        tr[2 * c] = df_mul(mre, ar[c]);
                        tr[2 * c + 1] = df_mul(df_neg(mim), ai[c]);
                        ti[2 * c] = df_mul(mre, ai[c]);
                        ti[2 * c + 1] = df_mul(mim, ar[c]);
                    }
                    const DF xr = df_sum<8>(tr), xi = df_sum<8>(ti);
                    v[idx[r]] = make_float4(xr.hi, xr.lo, xi.hi, xi.lo);
                }
            }
        }
    }
}

template <int GK, class OP>
__device__ __forceinline__ DF sweep_gen1_df(const float4 *lam, const float4 *bra, int E, const OP &o,
                                            const DF *g) {
    DF acc{0.0f, 0.0f};
    const uint32_t holes = o.gcm | (1u << o.gt);
    const int nfree = E >> __popc(holes);
    PairWalk w(holes, threadIdx.x, kSweepThreads);
    for (int f = threadIdx.x; f < nfree; f += kSweepThreads) {
        const int e0 = int(w.x | o.gcv), e1 = e0 | (1 << o.gt);
        w.step();
        const float4 ka = lam[e0], kb = lam[e1], ba = bra[e0], bb = bra[e1];
        const DF kv[4] = {DF{ka.x, ka.y}, DF{ka.z, ka.w}, DF{kb.x, kb.y}, DF{kb.z, kb.w}};
        const DF bv[4] = {DF{ba.x, ba.y}, DF{ba.z, ba.w}, DF{bb.x, bb.y}, DF{bb.z, bb.w}};
        acc = df_sum<2>({acc, gexp_df<GK>(g, bv, kv)});
    }
    return acc;
}

template <class OP>
__device__ __forceinline__ DF sweep_gen_df(const float4 *lam, const float4 *bra, int E, const OP &o,
                                           const SweepDF &d) {
    if (o.gkind == G_DENSE4) {
        DF acc{0.0f, 0.0f};
        const int qa = o.gt, qb = o.gq2;
        const uint32_t holes = (1u << qa) | (1u << qb);
        PairWalk w(holes, threadIdx.x, kSweepThreads);
        for (int f = threadIdx.x; f < (E >> 2); f += kSweepThreads) {
            const int e = int(w.x);
            w.step();
            const int idx[4] = {e, e | (1 << qb), e | (1 << qa), e | (1 << qa) | (1 << qb)};
            DF ar[4], ai[4];
#pragma unroll
            for (int c = 0; c < 4; c++) {
                const float4 x = lam[idx[c]];
                ar[c] = DF{x.x, x.y};
                ai[c] = DF{x.z, x.w};
            }
#pragma unroll
            for (int r = 0; r < 4; r++) {
                DF tr[8], ti[8];
#pragma unroll
                for (int c = 0; c < 4; c++) {
                    const DF gre = d.g[2 * (r * 4 + c)], gim = d.g[2 * (r * 4 + c) + 1];
                    tr[2 * c] = df_mul(gre, ar[c]);
                    tr[2 * c + 1] = df_mul(df_neg(gim), ai[c]);
                    ti[2 * c] = df_mul(gre, ai[c]);
                    ti[2 * c + 1] = df_mul(gim, ar[c]);
                }
                const DF yr = df_sum<8>(tr), yi = df_sum<8>(ti);
                const float4 b = bra[idx[r]];
                acc = df_sum<3>({acc, df_mul(DF{b.x, b.y}, yi), df_neg(df_mul(DF{b.z, b.w}, yr))});
            }
        }
        return acc;
    }
    switch (o.gkind) {
    case G_Z: return sweep_gen1_df<G_Z>(lam, bra, E, o, d.g);
    case G_X: return sweep_gen1_df<G_X>(lam, bra, E, o, d.g);
    case G_Y: return sweep_gen1_df<G_Y>(lam, bra, E, o, d.g);
    case G_P1: return sweep_gen1_df<G_P1>(lam, bra, E, o, d.g);
    default: return sweep_gen1_df<G_DENSE>(lam, bra, E, o, d.g);
    }
}

// The part of a SweepOp the float-float sweep reads (its first 48 bytes).
struct SweepHdr {
    int ukind, ubody, ut, uq2;
    uint32_t ucm, ucv;
    int gkind, gt, gq2;
    uint32_t gcm, gcv;
    int col;
};
static_assert(offsetof(SweepOp, col) + sizeof(int) == sizeof(SweepHdr) && offsetof(SweepOp, ukind) == 0,
              "SweepHdr is the head of SweepOp");
constexpr int kHdrWords = int(sizeof(SweepHdr) / 4), kDfWords = int(sizeof(SweepDF) / 4);
constexpr int kDescWords = kHdrWords + kDfWords;
static_assert(sizeof(SweepDF) % 4 == 0 && kDescWords <= kSweepThreads, "one descriptor word per thread");

__global__ void __launch_bounds__(kSweepThreads, 1)
    adjoint_sweep_df_kernel(const double2 *__restrict__ ket, double2 *const *__restrict__ bras, int n,
                            const SweepOp *__restrict__ ops, const SweepDF *__restrict__ dops, int nops,
                            double *__restrict__ jac, int K) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ DF red[kSweepThreads / 32];
    // the operations' descriptors pass through shared memory: operation i + 1's
    // is loaded while operation i runs (one word per thread)
    __shared__ __align__(16) uint32_t desc[2][kDescWords];
    auto desc_word = [&](int i, int w) -> uint32_t {
        return w < kHdrWords ? reinterpret_cast<const uint32_t *>(ops + i)[w]
                             : reinterpret_cast<const uint32_t *>(dops + i)[w - kHdrWords];
    };
    const int E = 1 << n;
    float4 *lam = reinterpret_cast<float4 *>(smem_raw);
    float4 *bra = lam + E;
    const int k = blockIdx.x;
    const double2 *src = bras[k];
    if (nops > 0 && threadIdx.x < kDescWords) desc[0][threadIdx.x] = desc_word(0, threadIdx.x);
    for (int e = threadIdx.x; e < E; e += kSweepThreads) {
        const double2 a = ket[e], b = src[e];
        const DF ar = df_from_double(a.x), ai = df_from_double(a.y), br = df_from_double(b.x), bi = df_from_double(b.y);
        lam[e] = make_float4(ar.hi, ar.lo, ai.hi, ai.lo);
        bra[e] = make_float4(br.hi, br.lo, bi.hi, bi.lo);
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int i = 0; i < nops; i++) {
        const bool pf = i + 1 < nops && threadIdx.x < kDescWords;
        const uint32_t next = pf ? desc_word(i + 1, threadIdx.x) : 0u;
        const SweepHdr &o = *reinterpret_cast<const SweepHdr *>(desc[i & 1]);
        const SweepDF &d = *reinterpret_cast<const SweepDF *>(desc[i & 1] + kHdrWords);
        if (o.col >= 0 && o.gkind != G_NONE) {
            DF v = sweep_gen_df(lam, bra, E, o, d);
#pragma unroll
            for (int s = 16; s > 0; s >>= 1) v = df_sum<2>({v, df_shfl_xor(v, s)});
            if (lane == 0) red[warp] = v;
            __syncthreads();
            if (threadIdx.x == 0) {
                DF t = red[0];
                for (int w = 1; w < kSweepThreads / 32; w++) t = df_sum<2>({t, red[w]});
                jac[size_t(o.col) * K + k] = df_to_double(t);
            }
            __syncthreads();
        }
        sweep_udag_df(lam, bra, E, o, d);
        if (pf) desc[(i + 1) & 1][threadIdx.x] = next;
        __syncthreads();
    }
}

// A complex128 state converted in place between complex128 and float-float
// (re.hi, im.hi, re.lo, im.lo) per amplitude.
__global__ void __launch_bounds__(256) state_to_ff_kernel(double2 *sv, uint64_t count) {
    const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
    for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < count; i += stride) {
        const double2 v = sv[i];
        const DF r = df_from_double(v.x), im = df_from_double(v.y);
        reinterpret_cast<float4 *>(sv)[i] = make_float4(r.hi, im.hi, r.lo, im.lo);
    }
}
__global__ void __launch_bounds__(256) state_from_ff_kernel(double2 *sv, uint64_t count) {
    const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
    for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < count; i += stride) {
        const float4 v = reinterpret_cast<const float4 *>(sv)[i];
        sv[i] = make_double2(df_to_double(DF{v.x, v.z}), df_to_double(DF{v.y, v.w}));
    }
}

template <class I>
static lgpu_status_t adjoint_block_t(lgpu_context_t ctx, void *ket, void *const *bras, uint32_t nbras, uint32_t n,
                                     const std::vector<int> &tile_bits, const lgpu_adj_block_step_t *steps,
                                     uint32_t nsteps, double *jac, uint32_t stride, bool c64, uint32_t ff_flags,
                                     cudaStream_t s) {
    const int k = int(tile_bits.size());
    std::vector<int> pos(n, -1);
    for (int q = 0; q < k; q++) pos[size_t(tile_bits[size_t(q)])] = q;
    int m = 0;
    while (m < k && tile_bits[size_t(m)] == m) m++;
    if (k - m > 6) return fail(LGPU_ERR_INVALID_ARG, "adjoint block: at most 6 tile bits above the low run");
    auto *p = new AdjBlockParams<I>();
    std::unique_ptr<AdjBlockParams<I>> guard(p);
    p->holes = make_holes(tile_bits);
    p->ntiles = I(uint64_t(1) << (n - uint32_t(k)));
    p->k = k;
    p->m = m;
    p->nb = int(nbras);
    p->in_ff = (ff_flags & LGPU_FF_IN) ? 1 : 0;
    p->out_ff = (ff_flags & LGPU_FF_OUT) ? 1 : 0;
    for (int h = 0; h < (1 << (k - m)); h++) {
        uint64_t o = 0;
        for (int q = m; q < k; q++)
            if ((h >> (q - m)) & 1) o |= uint64_t(1) << tile_bits[size_t(q)];
        p->hi_off[h] = I(o);
    }
    p->ket = static_cast<double2 *>(ket);
    for (uint32_t b = 0; b < nbras; b++) p->bras[b] = static_cast<double2 *>(bras[b]);
    std::vector<int> cols;
    p->nsteps = int(nsteps);
    for (uint32_t i = 0; i < nsteps; i++) {
        const lgpu_adj_block_step_t &a = steps[i];
        AStep &st = p->steps[i];
        st = AStep{};
        if (a.tgt < 0 || uint32_t(a.tgt) >= n || pos[size_t(a.tgt)] < 0)
            return fail(LGPU_ERR_INVALID_ARG, "adjoint block: target outside the tile");
        st.q = uint8_t(pos[size_t(a.tgt)]);
        if (a.nctrl < 0 || a.nctrl > 2) return fail(LGPU_ERR_INVALID_ARG, "adjoint block: at most 2 controls");
        for (int c = 0; c < a.nctrl; c++) {
            const int b = a.ctrl[c];
            if (b < 0 || uint32_t(b) >= n || b == a.tgt) return fail(LGPU_ERR_INVALID_ARG, "adjoint block: bad control");
            const uint32_t v = a.ctrl_val[c] ? 1u : 0u;
            if (pos[size_t(b)] >= 0) {
                st.in_mask |= 1u << pos[size_t(b)];
                st.in_val |= v << pos[size_t(b)];
            } else {
                st.out_mask |= uint64_t(1) << b;
                st.out_val |= uint64_t(v) << b;
            }
        }
        KConst kc[4];
        st.body = uint8_t(body_of_2x2_host(a.u, kc));
        st.pad = df_sign_diag_host(a.u) ? 1 : 0;  // sign flips instead of products
        for (int e = 0; e < 8; e++) {
            st.u[e] = df_split_host(a.u[e]);
            st.g[e] = df_split_host(a.g[e]);
        }
        if (a.gen_kind < 0) {
            st.gk = int8_t(G_NONE);
            st.slot = -1;
        } else {
            if (a.col < 0) return fail(LGPU_ERR_INVALID_ARG, "adjoint block: negative Jacobian column");
            const int gkd = gen_kind(a.g);
            st.gk = int8_t(gkd == G_NONE ? G_DENSE : gkd);
            st.slot = int32_t(cols.size());
            cols.push_back(a.col);
        }
    }
    p->nslots = int(cols.size());
    if (adj_phase_groups_enabled()) {
        // phase groups (lgpu_adj_plan.h): uncontrolled diagonal steps (RZ,
        // PhaseShift, or without gradient) gathered into one step each
        std::vector<AStep> in(p->steps, p->steps + nsteps);
        std::vector<AdjPlanStep> ps(nsteps);
        for (uint32_t i = 0; i < nsteps; i++) {
            const AStep &st = in[i];
            ps[i].q = st.q;
            ps[i].diagonal = st.body == B_DIAG || st.pad == 1;
            ps[i].groupable = st.body == B_DIAG && st.pad == 0 && st.in_mask == 0 && st.out_mask == 0 &&
                              (st.gk == G_NONE || st.gk == G_Z || st.gk == G_P1);
            ps[i].grad = st.gk != G_NONE;
        }
        const auto plan = plan_phase_groups(ps, kAdjGroupBits, kAdjGroupGrads);
        int ntab = 0;  // groups have two or more steps: at most kAdjBlockSteps / 2 tables
        for (size_t r = 0; r < plan.size(); r++) {
            const auto &mem = plan[r];
            if (mem.size() == 1) {
                p->steps[r] = in[mem[0]];
                continue;
            }
            AStep gs{};
            gs.pad = kAdjPhaseGroup;
            gs.gk = int8_t(G_NONE);
            gs.slot = ntab;  // its table in gtab
            for (uint32_t i : mem) gs.in_mask |= 1u << in[i].q;
            std::vector<int> bits;  // table positions, ascending
            for (int q = 0; q < 32; q++)
                if ((gs.in_mask >> q) & 1u) bits.push_back(q);
            for (int idx = 0; idx < (1 << kAdjGroupBits); idx++) {
                std::complex<double> t(1.0, 0.0);
                for (uint32_t i : mem) {
                    const double *u = steps[i].u;
                    const int rank = int(std::find(bits.begin(), bits.end(), int(in[i].q)) - bits.begin());
                    t *= ((idx >> rank) & 1) ? std::complex<double>(u[6], u[7]) : std::complex<double>(u[0], u[1]);
                }
                const DF re = df_split_host(t.real()), im = df_split_host(t.imag());
                p->gtab[ntab][idx] = make_float4(re.hi, re.lo, im.hi, im.lo);
            }
            for (uint32_t i : mem) {
                if (in[i].gk == G_NONE) continue;
                gs.gq[gs.ng] = in[i].q;
                gs.gkd[gs.ng] = in[i].gk;
                gs.gslot[gs.ng] = int16_t(in[i].slot);
                gs.ng++;
            }
            p->steps[r] = gs;
            ntab++;
        }
        p->nsteps = int(plan.size());
    }
    if (c64 && m < 1) return fail(LGPU_ERR_INVALID_ARG, "adjoint block: complex64 tiles need bit 0");
    const size_t tile_bytes = (size_t(1) << k) * (c64 ? 8 : 16);
    // tiles, the per-warp sums, then the phase-group table
    const size_t smem = (nbras + 1) * tile_bytes + size_t(std::max(p->nslots, 1)) * nbras * 8 * sizeof(DF) +
                        (size_t(16) << kAdjGroupBits);
    const int per_sm = std::max(1, std::min(3, int((220 * 1024) / smem)));
    const unsigned grid = unsigned(std::min<uint64_t>(uint64_t(p->ntiles), uint64_t(sm_count()) * per_sm));
    // scratch: [reduction counter, 256 B, untouched][columns][partials]
    const size_t cbytes = (sizeof(int) * std::max<size_t>(cols.size(), 1) + 255) & ~size_t(255);
    const size_t pbytes = sizeof(double) * size_t(grid) * std::max(p->nslots, 1) * nbras;
    void *scr = nullptr;
    LGPU_TRY(ctx_scratch(ctx, 256 + cbytes + pbytes, &scr));
    int *dcols = reinterpret_cast<int *>(static_cast<char *>(scr) + 256);
    p->partials = reinterpret_cast<double *>(static_cast<char *>(scr) + 256 + cbytes);
    if (!cols.empty()) {
        LGPU_CUDA_TRY(cudaMemcpyAsync(dcols, cols.data(), sizeof(int) * cols.size(), cudaMemcpyHostToDevice, s));
        LGPU_CUDA_TRY(cudaStreamSynchronize(s));  // the pageable source must outlive the copy
    }
    static std::atomic<size_t> attr1[64], attr2[64], attr3[64], attr4[64];
    if (c64 && nbras == 1) {
        LGPU_TRY(ensure_smem(reinterpret_cast<const void *>(adjoint_block_f32_kernel<I, 1>), smem, attr3));
        adjoint_block_f32_kernel<I, 1><<<grid, kAdjBlockThreads, smem, s>>>(*p);
    } else if (c64) {
        LGPU_TRY(ensure_smem(reinterpret_cast<const void *>(adjoint_block_f32_kernel<I, 2>), smem, attr4));
        adjoint_block_f32_kernel<I, 2><<<grid, kAdjBlockThreads, smem, s>>>(*p);
    } else if (nbras == 1) {
        LGPU_TRY(ensure_smem(reinterpret_cast<const void *>(adjoint_block_kernel<I, 1>), smem, attr1));
        adjoint_block_kernel<I, 1><<<grid, kAdjBlockThreads, smem, s>>>(*p);
    } else {
        LGPU_TRY(ensure_smem(reinterpret_cast<const void *>(adjoint_block_kernel<I, 2>), smem, attr2));
        adjoint_block_kernel<I, 2><<<grid, kAdjBlockThreads, smem, s>>>(*p);
    }
    LGPU_CHECK_LAUNCH();
    if (!cols.empty()) {
        const int total = p->nslots * int(nbras);
        adjoint_block_reduce<<<(total + 3) / 4, 128, 0, s>>>(p->partials, int(grid), p->nslots, int(nbras), dcols, jac,
                                                             int(stride));
        LGPU_CHECK_LAUNCH();
    }
    return LGPU_OK;
}

}  // namespace lgpu

using namespace lgpu;

extern "C" {

lgpu_status_t lgpu_adjoint_step(lgpu_context_t ctx, void *ket, void *const *bras, uint32_t nbras, uint32_t n,
                                lgpu_dtype_t dt, uint32_t w, const int32_t *bits, const double *gen,
                                const double *udag, int apply_udag, double *out_dev, lgpu_stream_t stream) {
    LGPU_TRY(check_state(ket, n, dt));
    if (nbras && !bras) return fail(LGPU_ERR_INVALID_ARG, "bras is null");
    for (uint32_t k = 0; k < nbras; k++) LGPU_TRY(check_state(bras[k], n, dt));
    if (w < 1 || w > 4 || w > n) return fail(LGPU_ERR_INVALID_ARG, "adjoint step: 1 to 4 bits");
    if (gen && nbras && !out_dev) return fail(LGPU_ERR_INVALID_ARG, "adjoint step: output is null");
    if (apply_udag && !udag) return fail(LGPU_ERR_INVALID_ARG, "adjoint step: U^dag is null");
    std::vector<int> b;
    LGPU_TRY(check_bits(n, w, bits, "adjoint", &b));
    std::vector<int> srt(b);
    std::sort(srt.begin(), srt.end());
    if (std::adjacent_find(srt.begin(), srt.end()) != srt.end())
        return fail(LGPU_ERR_INVALID_ARG, "repeated bit");
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    if (dt == LGPU_C128)
        return n <= 32 ? adjoint_dispatch<double, uint32_t>(ctx, ket, bras, nbras, n, b, gen, udag, apply_udag, out_dev, s)
                       : adjoint_dispatch<double, uint64_t>(ctx, ket, bras, nbras, n, b, gen, udag, apply_udag, out_dev, s);
    return n <= 32 ? adjoint_dispatch<float, uint32_t>(ctx, ket, bras, nbras, n, b, gen, udag, apply_udag, out_dev, s)
                   : adjoint_dispatch<float, uint64_t>(ctx, ket, bras, nbras, n, b, gen, udag, apply_udag, out_dev, s);
}


lgpu_status_t lgpu_adjoint_block_ff(lgpu_context_t ctx, void *ket, void *const *bras, uint32_t nbras, uint32_t n,
                                    lgpu_dtype_t dt, uint32_t k, const int32_t *tile_bits,
                                    const lgpu_adj_block_step_t *steps, uint32_t nsteps, double *jac_dev,
                                    uint32_t jac_stride, uint32_t ff_flags, lgpu_stream_t stream) {
    LGPU_TRY(check_state(ket, n, dt));
    if (nbras < 1 || nbras > uint32_t(kAdjBlockBras) || !bras)
        return fail(LGPU_ERR_INVALID_ARG, "adjoint block: 1 or 2 bras");
    for (uint32_t b = 0; b < nbras; b++) LGPU_TRY(check_state(bras[b], n, dt));
    if (ff_flags & ~uint32_t(LGPU_FF_IN | LGPU_FF_OUT)) return fail(LGPU_ERR_INVALID_ARG, "adjoint block: unknown flags");
    if (ff_flags && dt != LGPU_C128)
        return fail(LGPU_ERR_INVALID_ARG, "adjoint block: float-float states are complex128 only");
    if (nsteps == 0) {
        // nothing to apply; the states still take the requested form
        if ((ff_flags & LGPU_FF_IN) != 0 && (ff_flags & LGPU_FF_OUT) == 0) {
            LGPU_TRY(lgpu_state_ff(ket, n, 0, stream));
            for (uint32_t b = 0; b < nbras; b++) LGPU_TRY(lgpu_state_ff(bras[b], n, 0, stream));
        } else if ((ff_flags & LGPU_FF_IN) == 0 && (ff_flags & LGPU_FF_OUT) != 0) {
            LGPU_TRY(lgpu_state_ff(ket, n, 1, stream));
            for (uint32_t b = 0; b < nbras; b++) LGPU_TRY(lgpu_state_ff(bras[b], n, 1, stream));
        }
        return LGPU_OK;
    }
    if (!steps || nsteps > uint32_t(kAdjBlockSteps)) return fail(LGPU_ERR_INVALID_ARG, "adjoint block: 1 to 48 steps");
    if (k < 1 || k > 11 || k > n) return fail(LGPU_ERR_INVALID_ARG, "adjoint block: tile of 1 to 11 bits");
    if (!jac_dev || jac_stride < nbras) return fail(LGPU_ERR_INVALID_ARG, "adjoint block: Jacobian output");
    std::vector<int> tb;
    LGPU_TRY(check_bits(n, k, tile_bits, "tile", &tb));
    std::sort(tb.begin(), tb.end());
    if (std::adjacent_find(tb.begin(), tb.end()) != tb.end())
        return fail(LGPU_ERR_INVALID_ARG, "tile bits must be distinct");
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const bool c64 = dt == LGPU_C64;
    return n <= 32 ? adjoint_block_t<uint32_t>(ctx, ket, bras, nbras, n, tb, steps, nsteps, jac_dev, jac_stride, c64,
                                               ff_flags, s)
                   : adjoint_block_t<uint64_t>(ctx, ket, bras, nbras, n, tb, steps, nsteps, jac_dev, jac_stride, c64,
                                               ff_flags, s);
}

lgpu_status_t lgpu_adjoint_block(lgpu_context_t ctx, void *ket, void *const *bras, uint32_t nbras, uint32_t n,
                                 lgpu_dtype_t dt, uint32_t k, const int32_t *tile_bits,
                                 const lgpu_adj_block_step_t *steps, uint32_t nsteps, double *jac_dev,
                                 uint32_t jac_stride, lgpu_stream_t stream) {
    return lgpu_adjoint_block_ff(ctx, ket, bras, nbras, n, dt, k, tile_bits, steps, nsteps, jac_dev, jac_stride, 0,
                                 stream);
}

lgpu_status_t lgpu_state_ff(void *sv, uint32_t n, int to_ff, lgpu_stream_t stream) {
    LGPU_TRY(check_state(sv, n, LGPU_C128));
    const uint64_t count = uint64_t(1) << n;
    const unsigned g = grid_for(count, 256, 8, 8);
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    if (to_ff)
        state_to_ff_kernel<<<g, 256, 0, s>>>(static_cast<double2 *>(sv), count);
    else
        state_from_ff_kernel<<<g, 256, 0, s>>>(static_cast<double2 *>(sv), count);
    LGPU_CHECK_LAUNCH();
    return LGPU_OK;
}

uint32_t lgpu_adjoint_sweep_max_qubits(lgpu_dtype_t dt) { return dt == LGPU_C128 ? 12u : 13u; }

lgpu_status_t lgpu_adjoint_sweep_small(lgpu_context_t ctx, const void *ket, void *const *bras, uint32_t nbras,
                                       uint32_t n, lgpu_dtype_t dt, const lgpu_adj_op_t *ops, uint32_t nops,
                                       double *jac_dev, lgpu_stream_t stream) {
    LGPU_TRY(check_state(ket, n, dt));
    if (n > lgpu_adjoint_sweep_max_qubits(dt))
        return fail(LGPU_ERR_INVALID_ARG, "adjoint sweep: the state does not fit in shared memory");
    if (nbras == 0) return LGPU_OK;
    if (!bras || !jac_dev || (nops && !ops)) return fail(LGPU_ERR_INVALID_ARG, "adjoint sweep: null argument");
    for (uint32_t k = 0; k < nbras; k++) LGPU_TRY(check_state(bras[k], n, dt));
    std::vector<SweepOp> host(std::max<uint32_t>(nops, 1));
    for (uint32_t i = 0; i < nops; i++) LGPU_TRY(sweep_op_of(ops[i], n, &host[i]));
    // scratch: [reduction counter, 256 B, left untouched][bra pointers, 256-byte aligned][ops]
    const size_t pbytes = (sizeof(void *) * nbras + 255) & ~size_t(255);
    void *p = nullptr;
    LGPU_TRY(ctx_scratch(ctx, 256 + pbytes + sizeof(SweepOp) * host.size(), &p));
    void **dbras = reinterpret_cast<void **>(static_cast<char *>(p) + 256);
    auto *dops = reinterpret_cast<SweepOp *>(static_cast<char *>(p) + 256 + pbytes);
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    LGPU_CUDA_TRY(cudaMemcpyAsync(dbras, bras, sizeof(void *) * nbras, cudaMemcpyHostToDevice, s));
    if (nops) LGPU_CUDA_TRY(cudaMemcpyAsync(dops, host.data(), sizeof(SweepOp) * nops, cudaMemcpyHostToDevice, s));
    // the pageable source vectors must outlive the copies
    LGPU_CUDA_TRY(cudaStreamSynchronize(s));
    if (dt == LGPU_C128 && f64_mode() == 1 && fused_df_enabled()) {
        // float-float copies of the coefficients, after the ops in the scratch
        std::vector<SweepDF> hd(host.size());
        for (uint32_t i = 0; i < nops; i++) {
            for (int e = 0; e < 32; e++) {
                hd[i].u[e] = df_split_host(host[i].u[e]);
                hd[i].g[e] = df_split_host(host[i].g[e]);
            }
            hd[i].sign_diag = host[i].ukind == U_ONE && df_sign_diag_host(host[i].u) ? 1 : 0;
        }
        const size_t obytes = (sizeof(SweepOp) * host.size() + 255) & ~size_t(255);
        LGPU_TRY(ctx_scratch(ctx, 256 + pbytes + obytes + sizeof(SweepDF) * hd.size(), &p));
        dbras = reinterpret_cast<void **>(static_cast<char *>(p) + 256);
        dops = reinterpret_cast<SweepOp *>(static_cast<char *>(p) + 256 + pbytes);
        auto *ddf = reinterpret_cast<SweepDF *>(static_cast<char *>(p) + 256 + pbytes + obytes);
        LGPU_CUDA_TRY(cudaMemcpyAsync(dbras, bras, sizeof(void *) * nbras, cudaMemcpyHostToDevice, s));
        if (nops) {
            LGPU_CUDA_TRY(cudaMemcpyAsync(dops, host.data(), sizeof(SweepOp) * nops, cudaMemcpyHostToDevice, s));
            LGPU_CUDA_TRY(cudaMemcpyAsync(ddf, hd.data(), sizeof(SweepDF) * nops, cudaMemcpyHostToDevice, s));
        }
        LGPU_CUDA_TRY(cudaStreamSynchronize(s));
        const size_t smem = 2 * (size_t(1) << n) * sizeof(double2);
        static std::atomic<size_t> attr[64];
        LGPU_TRY(ensure_smem(reinterpret_cast<const void *>(adjoint_sweep_df_kernel), smem, attr));
        adjoint_sweep_df_kernel<<<nbras, kSweepThreads, smem, s>>>(static_cast<const double2 *>(ket),
                                                                   reinterpret_cast<double2 *const *>(dbras), int(n),
                                                                   dops, ddf, int(nops), jac_dev, int(nbras));
        LGPU_CHECK_LAUNCH();
        return LGPU_OK;
    }
    if (dt == LGPU_C128)
        return f64_mode() == 1 ? sweep_launch<double, true>(ket, dbras, nbras, n, dops, nops, jac_dev, s)
                               : sweep_launch<double, false>(ket, dbras, nbras, n, dops, nops, jac_dev, s);
    return sweep_launch<float, false>(ket, dbras, nbras, n, dops, nops, jac_dev, s);
}

}  // extern "C"
