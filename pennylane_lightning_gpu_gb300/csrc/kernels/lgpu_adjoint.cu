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
    const unsigned g = reduce_grid(uint64_t(ngroups));
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
    case 1: return adjoint_t<T, I, 1>(ctx, ket, bras, nbras, n, bits, gen, udag, apply_udag, out_dev, s);
    case 2: return adjoint_t<T, I, 2>(ctx, ket, bras, nbras, n, bits, gen, udag, apply_udag, out_dev, s);
    case 3: return adjoint_t<T, I, 3>(ctx, ket, bras, nbras, n, bits, gen, udag, apply_udag, out_dev, s);
    case 4: return adjoint_t<T, I, 4>(ctx, ket, bras, nbras, n, bits, gen, udag, apply_udag, out_dev, s);
    default: return fail(LGPU_ERR_INVALID_ARG, "adjoint step: 1 to 4 bits");
    }
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

}  // extern "C"
