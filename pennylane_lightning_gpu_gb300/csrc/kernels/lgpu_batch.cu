// liblgpu_gb300: batched execution of many independent circuits in one
// persistent launch.
//
//  * bprep_kernel   builds every gate's matrix (and, for complex128, the
//                   integer-pipe multiplier constants) from a device parameter
//                   buffer, so that a captured CUDA graph can be replayed with
//                   new parameters by copying only the parameter buffer.
//  * batch_kernel   persistent CTAs take circuits from an atomic work queue
//                   (host orders them largest first).  A circuit with
//                   n <= kmax qubits lives entirely in shared memory; a larger
//                   one is streamed through shared-memory tiles block by block
//                   (the host fuses its gates into blocks whose targets fit a
//                   tile) using a per-CTA scratch state in global memory.  The
//                   observable (a sum of Pauli words) is evaluated on the
//                   tiles of the last block and reduced inside the CTA, so each
//                   result is written by exactly one CTA in a fixed order.
#include "lgpu_bodies.cuh"
#include "lgpu_df2.cuh"
#include "lgpu_df64.cuh"
#include "lgpu_f64emu.cuh"
#include "lgpu_internal.cuh"

namespace lgpu {

// body kinds
enum BKind : uint8_t { BK_DENSE1 = 0, BK_DIAG1, BK_X1, BK_REAL1, BK_RXLIKE1, BK_DENSE2, BK_SWAP2, BK_CHAINED };
constexpr uint32_t kChainHead = 2u;  // flags bit 1: the next q1 gates (BK_CHAINED) fold into this one
// parameter kinds (matrix built on device)
enum PKind : uint8_t { PK_NONE = 0, PK_RX, PK_RY, PK_RZ, PK_PHASE, PK_ROT, PK_ISINGXX, PK_ISINGYY, PK_ISINGZZ };

static_assert(sizeof(lgpu_bgate_t) == 40, "lgpu_bgate_t layout");

// ---------------------------------------------------------------------------
// Matrix preparation
// ---------------------------------------------------------------------------
// Matrix of one gate into m (8 doubles for 1 target, 32 for 2): from the
// parameters for parametric gates, from the pool for fixed ones.
__device__ void bgate_matrix(const lgpu_bgate_t &g, const double *__restrict__ params, const double *pool, double *m) {
    const bool adj = (g.flags & 1u) != 0;
    if (g.pkind == PK_NONE) {
        const int cnt = (g.kind == BK_DENSE2 || g.kind == BK_SWAP2) ? 32 : 8;
        for (int e = 0; e < cnt; e++) m[e] = pool[g.mat + e];
        return;
    }
    const double th0 = params[g.param];
    const double th = adj ? -th0 : th0;
    if (g.pkind == PK_RX || g.pkind == PK_RY || g.pkind == PK_RZ || g.pkind == PK_PHASE) {
        double s, c;
        if (g.pkind == PK_PHASE) {
            sincos(th, &s, &c);
            m[0] = 1; m[1] = 0; m[2] = 0; m[3] = 0; m[4] = 0; m[5] = 0; m[6] = c; m[7] = s;
        } else {
            sincos(0.5 * th, &s, &c);
            if (g.pkind == PK_RX) {
                m[0] = c; m[1] = 0; m[2] = 0; m[3] = -s; m[4] = 0; m[5] = -s; m[6] = c; m[7] = 0;
            } else if (g.pkind == PK_RY) {
                m[0] = c; m[1] = 0; m[2] = -s; m[3] = 0; m[4] = s; m[5] = 0; m[6] = c; m[7] = 0;
            } else {
                m[0] = c; m[1] = -s; m[2] = 0; m[3] = 0; m[4] = 0; m[5] = 0; m[6] = c; m[7] = s;
            }
        }
    } else if (g.pkind == PK_ROT) {
        // Rot(phi, theta, omega) = RZ(omega) RY(theta) RZ(phi); adjoint = Rot(-omega, -theta, -phi)
        double phi = params[g.param], theta = params[g.param + 1], omega = params[g.param + 2];
        if (adj) {
            const double t = phi;
            phi = -omega;
            theta = -theta;
            omega = -t;
        }
        double cs, sn, cp, sp, cm, sm;
        sincos(0.5 * theta, &sn, &cs);
        sincos(0.5 * (phi + omega), &sp, &cp);
        sincos(0.5 * (phi - omega), &sm, &cm);
        m[0] = cs * cp; m[1] = -cs * sp;
        m[2] = -sn * cm; m[3] = -sn * sm;
        m[4] = sn * cm; m[5] = -sn * sm;
        m[6] = cs * cp; m[7] = cs * sp;
    } else {
        double s, c;
        sincos(0.5 * th, &s, &c);
        for (int e = 0; e < 32; e++) m[e] = 0.0;
        if (g.pkind == PK_ISINGZZ) {
            // diag(e^{-i t/2}, e^{i t/2}, e^{i t/2}, e^{-i t/2})
            m[0] = c; m[1] = -s; m[10] = c; m[11] = s; m[20] = c; m[21] = s; m[30] = c; m[31] = -s;
        } else {
            const double corner = g.pkind == PK_ISINGXX ? -s : s;  // YY: +i s at (0,3),(3,0)
            for (int d = 0; d < 4; d++) m[2 * (d * 4 + d)] = c;
            m[2 * (0 * 4 + 3) + 1] = corner;
            m[2 * (3 * 4 + 0) + 1] = corner;
            m[2 * (1 * 4 + 2) + 1] = -s;
            m[2 * (2 * 4 + 1) + 1] = -s;
        }
    }
}

// complex128 batches run in float-float (the same switch as the fused blocks).
static bool batch_df() { return f64_mode() == 1 && fused_df_enabled() != 0; }

// mode: 0 = complex128 with integer-pipe constants, 1 = complex64 (float
// copy), 2 = complex128 in float-float (the (hi, lo) pairs of a 1-target
// matrix at pool + mat + 8).
__global__ void bprep_kernel(const lgpu_bgate_t *__restrict__ gates, uint64_t ngates, const double *__restrict__ params,
                             double *__restrict__ pool, int mode) {
    const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
    for (uint64_t gi = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; gi < ngates; gi += stride) {
        const lgpu_bgate_t g = gates[gi];
        if (g.kind == BK_CHAINED) continue;  // folded into its chain head
        double *m = pool + g.mat;
        if (g.flags & kChainHead) {
            // product M_q1 ... M_2 M_1 of the run of 1-target gates on one bit
            // recorded after the head (their own slots stay untouched, so a
            // replay with new parameters rebuilds it)
            double a[8] = {1, 0, 0, 0, 0, 0, 1, 0}, b[8];
            for (uint32_t c = 1; c <= g.q1; c++) {
                bgate_matrix(gates[gi + c], params, pool, b);
                double r[8];
                for (int i = 0; i < 2; i++)
                    for (int j = 0; j < 2; j++) {
                        double re = 0, im = 0;
                        for (int k = 0; k < 2; k++) {
                            const double br = b[2 * (i * 2 + k)], bi = b[2 * (i * 2 + k) + 1];
                            const double ar = a[2 * (k * 2 + j)], ai = a[2 * (k * 2 + j) + 1];
                            re += br * ar - bi * ai;
                            im += br * ai + bi * ar;
                        }
                        r[2 * (i * 2 + j)] = re;
                        r[2 * (i * 2 + j) + 1] = im;
                    }
                for (int e = 0; e < 8; e++) a[e] = r[e];
            }
            for (int e = 0; e < 8; e++) m[e] = a[e];
        } else if (g.pkind != PK_NONE) {
            bgate_matrix(g, params, pool, m);
        }
        // (fixed matrices arrive from the host already in their final, adjointed form)
        if (mode == 2) {
            if (g.kind < BK_DENSE2) {
                DF *d = reinterpret_cast<DF *>(m + 8);
                for (int e = 0; e < 8; e++) d[e] = df_from_double(m[e]);
            }
            continue;
        }
        if (mode == 1) {
            // complex64: a float copy of the matrix (1q: pool + mat + 8, 2q: pool + mat + 32)
            float *f = reinterpret_cast<float *>(m + (g.kind < BK_DENSE2 ? 8 : 32));
            const int cnt = g.kind < BK_DENSE2 ? 8 : 32;
            for (int e = 0; e < cnt; e++) f[e] = float(m[e]);
            continue;
        }
        // integer-pipe multiplier constants for the complex128 structured bodies
        if (g.kind < BK_DENSE2) {
            KConst *k = reinterpret_cast<KConst *>(m + 8);
            if (g.kind == BK_DIAG1) {
                k[0] = make_kconst(-m[1]); k[1] = make_kconst(m[1]); k[2] = make_kconst(-m[7]); k[3] = make_kconst(m[7]);
            } else if (g.kind == BK_REAL1) {
                k[0] = make_kconst(m[2]); k[1] = make_kconst(m[4]); k[2] = make_kconst(0.0); k[3] = make_kconst(0.0);
            } else if (g.kind == BK_RXLIKE1) {
                k[0] = make_kconst(-m[3]); k[1] = make_kconst(m[3]); k[2] = make_kconst(-m[5]); k[3] = make_kconst(m[5]);
            } else if (g.kind == BK_DENSE1) {
                k[0] = make_kconst(m[1]); k[1] = make_kconst(m[3]); k[2] = make_kconst(m[5]); k[3] = make_kconst(m[7]);
            }
        }
    }
}

// ---------------------------------------------------------------------------
// In-shared-memory gate application
// ---------------------------------------------------------------------------
// Matrix coefficients of a 1-target gate in the state's precision: the
// complex64 copy (floats at pool + mat + 8) is written by bprep_kernel, so no
// double->float conversion (an FP64-pipe instruction) runs per amplitude.
template <class T, bool EMU>
__device__ __forceinline__ void load_coef1(const double *pool, uint32_t mat, T (&m)[8], KConst (&k)[4]) {
    if constexpr (sizeof(T) == 4) {
        const float4 *f = reinterpret_cast<const float4 *>(pool + mat + 8);
        const float4 u = f[0], v = f[1];
        m[0] = u.x; m[1] = u.y; m[2] = u.z; m[3] = u.w;
        m[4] = v.x; m[5] = v.y; m[6] = v.z; m[7] = v.w;
#pragma unroll
        for (int i = 0; i < 4; i++) k[i] = KConst{};
    } else {
        const double2 *d = reinterpret_cast<const double2 *>(pool + mat);
#pragma unroll
        for (int i = 0; i < 4; i++) {
            const double2 v = d[i];
            m[2 * i] = v.x;
            m[2 * i + 1] = v.y;
        }
        const KConst *kc = reinterpret_cast<const KConst *>(pool + mat + 8);
#pragma unroll
        for (int i = 0; i < 4; i++) k[i] = EMU ? kc[i] : KConst{};
    }
}

template <class T, int BODY, bool EMU>
__device__ __forceinline__ void batch_pairs(cplx_t<T> *tile, int E, int q, uint32_t cmask, uint32_t cval,
                                            const double *pool, uint32_t mat) {
    using C = cplx_t<T>;
    T m[8];
    KConst k[4];
    load_coef1<T, EMU>(pool, mat, m, k);
    const uint32_t holes = cmask | (1u << q);
    const int nfree = E >> __popc(holes);
    PairWalk w(holes, threadIdx.x, blockDim.x);
#pragma unroll 2
    for (int f = threadIdx.x; f < nfree; f += blockDim.x) {
        const int e0 = int(w.x | cval);
        const int e1 = e0 | (1 << q);
        w.step();
        C a0 = tile[e0], a1 = tile[e1];
        body1_sel<T, BODY, EMU>(m, k, a0, a1);
        tile[e0] = a0;
        tile[e1] = a1;
    }
}

// complex128 in float-float: the tile holds float4 (re.hi, im.hi, re.lo,
// im.lo) per amplitude, in the slot of its double2; the bodies run as paired
// float-float lanes (re, im) (lgpu_df2.cuh).
template <int BODY>
__device__ __forceinline__ void batch_pairs_df(float4 *tile, int E, int q, uint32_t cmask, uint32_t cval,
                                               const DF *mp) {
    DF2 c[8];
    if constexpr (BODY != B_PERM) df2_coeffs(mp, c);
    const uint32_t holes = cmask | (1u << q);
    const int nfree = E >> __popc(holes);
    PairWalk w(holes, threadIdx.x, blockDim.x);
#pragma unroll 2
    for (int f = threadIdx.x; f < nfree; f += blockDim.x) {
        const int e0 = int(w.x | cval);
        const int e1 = e0 | (1 << q);
        w.step();
        float4 a = tile[e0], b = tile[e1];
        if constexpr (BODY == B_PERM) {
            tile[e0] = b;
            tile[e1] = a;
        } else {
            DF2 x{f2_pack(a.x, a.y), f2_pack(a.z, a.w)}, y{f2_pack(b.x, b.y), f2_pack(b.z, b.w)};
            body1_df2<BODY>(c, x, y);
            tile[e0] = make_float4(f2_x(x.hi), f2_y(x.hi), f2_x(x.lo), f2_y(x.lo));
            tile[e1] = make_float4(f2_x(y.hi), f2_y(y.hi), f2_x(y.lo), f2_y(y.lo));
        }
    }
}

__device__ __forceinline__ void tile_gate_df(float4 *tile, int E, const lgpu_bgate_t &g, const double *pool) {
    if (g.kind < BK_DENSE2) {
        const int q = g.q0;
        const DF *m = reinterpret_cast<const DF *>(pool + g.mat + 8);
        switch (g.kind) {
        case BK_DIAG1: batch_pairs_df<B_DIAG>(tile, E, q, g.cmask, g.cval, m); break;
        case BK_X1: batch_pairs_df<B_PERM>(tile, E, q, g.cmask, g.cval, m); break;
        case BK_REAL1: batch_pairs_df<B_REAL>(tile, E, q, g.cmask, g.cval, m); break;
        case BK_RXLIKE1: batch_pairs_df<B_RXLIKE>(tile, E, q, g.cmask, g.cval, m); break;
        default: batch_pairs_df<B_DENSE>(tile, E, q, g.cmask, g.cval, m); break;
        }
        return;
    }
    const int qa = g.q0, qb = g.q1;
    const uint32_t holes = g.cmask | (1u << qa) | (1u << qb);
    const int nfree = E >> __popc(holes);
    PairWalk w(holes, threadIdx.x, blockDim.x);
    const double *mm = pool + g.mat;  // 4x4 doubles, split per use (2-target gates are rare)
    for (int f = threadIdx.x; f < nfree; f += blockDim.x) {
        const int e = int(w.x | g.cval);
        w.step();
        const int idx[4] = {e, e | (1 << qb), e | (1 << qa), e | (1 << qa) | (1 << qb)};
        if (g.kind == BK_SWAP2) {
            const float4 t = tile[idx[1]];
            tile[idx[1]] = tile[idx[2]];
            tile[idx[2]] = t;
            continue;
        }
        DF ar[4], ai[4];
#pragma unroll
        for (int c = 0; c < 4; c++) {
            const float4 v = tile[idx[c]];  // (re.hi, im.hi, re.lo, im.lo)
            ar[c] = DF{v.x, v.z};
            ai[c] = DF{v.y, v.w};
        }
#pragma unroll
        for (int row = 0; row < 4; row++) {
            DF tr[8], ti[8];
#pragma unroll
            for (int c = 0; c < 4; c++) {
                const DF mre = df_from_double(mm[2 * (row * 4 + c)]), mim = df_from_double(mm[2 * (row * 4 + c) + 1]);
                tr[2 * c] = df_mul(mre, ar[c]);
                tr[2 * c + 1] = df_mul(df_neg(mim), ai[c]);
                ti[2 * c] = df_mul(mre, ai[c]);
                ti[2 * c + 1] = df_mul(mim, ar[c]);
            }
            const DF xr = df_sum<8>(tr), xi = df_sum<8>(ti);
            tile[idx[row]] = make_float4(xr.hi, xi.hi, xr.lo, xi.lo);
        }
    }
}

// float-float tile -> complex128, in place (all threads; the caller
// synchronises afterwards).
__device__ __forceinline__ void tile_from_df(void *tile, int E) {
    for (int e = threadIdx.x; e < E; e += blockDim.x) {
        const float4 v = reinterpret_cast<const float4 *>(tile)[e];
        reinterpret_cast<double2 *>(tile)[e] = make_double2(df_to_double(DF{v.x, v.z}), df_to_double(DF{v.y, v.w}));
    }
}

// Apply one gate to the tile in shared memory (all threads; the caller
// synchronises afterwards).
template <class T, bool EMU>
__device__ __forceinline__ void tile_gate(cplx_t<T> *tile, int E, const lgpu_bgate_t &g, const double *pool) {
    using C = cplx_t<T>;
    if (g.kind < BK_DENSE2) {
        const int q = g.q0;
        switch (g.kind) {
        case BK_DIAG1: batch_pairs<T, B_DIAG, EMU>(tile, E, q, g.cmask, g.cval, pool, g.mat); break;
        case BK_X1: batch_pairs<T, B_PERM, EMU>(tile, E, q, g.cmask, g.cval, pool, g.mat); break;
        case BK_REAL1: batch_pairs<T, B_REAL, EMU>(tile, E, q, g.cmask, g.cval, pool, g.mat); break;
        case BK_RXLIKE1: batch_pairs<T, B_RXLIKE, EMU>(tile, E, q, g.cmask, g.cval, pool, g.mat); break;
        default: batch_pairs<T, B_DENSE, EMU>(tile, E, q, g.cmask, g.cval, pool, g.mat); break;
        }
        return;
    }
    const int qa = g.q0, qb = g.q1;
    const uint32_t holes = g.cmask | (1u << qa) | (1u << qb);
    const int nfree = E >> __popc(holes);
    PairWalk w(holes, threadIdx.x, blockDim.x);
    // 4x4 coefficients: doubles at pool + mat, the complex64 copy (floats) at pool + mat + 32
    const T *mm = sizeof(T) == 4 ? reinterpret_cast<const T *>(pool + g.mat + 32)
                                 : reinterpret_cast<const T *>(pool + g.mat);
    for (int f = threadIdx.x; f < nfree; f += blockDim.x) {
        const int e = int(w.x | g.cval);
        w.step();
        const int i0 = e, i1 = e | (1 << qb), i2 = e | (1 << qa), i3 = e | (1 << qa) | (1 << qb);
        if (g.kind == BK_SWAP2) {
            const C t = tile[i1];
            tile[i1] = tile[i2];
            tile[i2] = t;
            continue;
        }
        const C a[4] = {tile[i0], tile[i1], tile[i2], tile[i3]};
        C r[4];
#pragma unroll
        for (int row = 0; row < 4; row++) {
            T xr = 0, xi = 0;
#pragma unroll
            for (int c = 0; c < 4; c++) {
                const T mr = mm[2 * (row * 4 + c)], mi = mm[2 * (row * 4 + c) + 1];
                xr = fmaT(mr, a[c].x, fmaT(-mi, a[c].y, xr));
                xi = fmaT(mr, a[c].y, fmaT(mi, a[c].x, xi));
            }
            r[row] = mk<T>(xr, xi);
        }
        tile[i0] = r[0];
        tile[i1] = r[1];
        tile[i2] = r[2];
        tile[i3] = r[3];
    }
}

// ---------------------------------------------------------------------------
// Observable on a tile
// ---------------------------------------------------------------------------
// Term t contributes Re((cr + i ci) sum_e s_t(e) conj(a_e) a_{e^F}), F its flip
// mask in tile positions and s_t(e) = (-1)^popc(g(e^F) & sign_t) with g the
// global index.  With L_t the sign mask in tile positions,
//   popc(g(e^F) & sign) = popc(base & sign) + popc(F & L_t) + popc(e & L_t)  (mod 2).
// Thread `slot` owns e = slot + S*i (i = 0..7, S = E/8); the sign over i is
// (-1)^popc(i & h_t), h_t = L_t >> log2 S, so the eight products of one flip
// group go through one 8-point Walsh-Hadamard transform and each term then
// costs a select and one multiply-add instead of a pass over the tile.
// s_lm[t] = L_t | popc(F & L_t) << 31 and s_c[t] = (cr, ci) are per block.
constexpr uint32_t kObsTermsCached = 1024;

template <class T>
__device__ __forceinline__ double tile_obs(const cplx_t<T> *tile, int k, const lgpu_bterm_t *terms, uint32_t nterms,
                                           uint64_t base, const uint32_t *s_lm, const cplx_t<T> *s_c) {
    using A = T;
    const int lgS = k - 3, S = 1 << lgS;
    A acc = 0;
    for (int slot = threadIdx.x; slot < S; slot += blockDim.x) {
        uint32_t t0 = 0;
        while (t0 < nterms) {
            const uint32_t F = terms[t0].tflip;
            uint32_t t1 = t0 + 1;
            while (t1 < nterms && terms[t1].tflip == F) t1++;
            const int fs = int(F) & (S - 1), fh = int(F) >> lgS;
            A xr[8], xi[8];
#pragma unroll
            for (int i = 0; i < 8; i++) {
                const cplx_t<T> a = tile[slot + S * i];
                if (F) {
                    const cplx_t<T> b = tile[(slot ^ fs) + S * (i ^ fh)];
                    xr[i] = a.x * b.x + a.y * b.y;
                    xi[i] = a.x * b.y - a.y * b.x;
                } else {
                    xr[i] = a.x * a.x + a.y * a.y;
                    xi[i] = A(0);
                }
            }
            wht8(xr);
            if (F) wht8(xi);
            for (uint32_t t = t0; t < t1; t++) {
                const uint32_t lm = s_lm[t];
                const uint32_t L = lm & 0x7fffffffu;
                const int par =
                    (__popc(uint32_t(slot) & L & uint32_t(S - 1)) + __popcll(base & terms[t].sign) + int(lm >> 31)) & 1;
                const int h = int(L >> lgS) & 7;
                const cplx_t<T> c = s_c[t];
                A v = c.x * sel8(xr, h);
                if (F) v -= c.y * sel8(xi, h);
                acc += par ? -v : v;
            }
            t0 = t1;
        }
    }
    return double(acc);
}

// Direct form for tiles of fewer than 8 amplitudes or more terms than cached.
template <class T>
__device__ __forceinline__ double tile_obs_direct(const cplx_t<T> *tile, int E, const lgpu_bterm_t *terms,
                                                  uint32_t nterms, uint64_t base, int m, const uint64_t *hi_off) {
    double acc = 0.0;
    const int lowmask = (1 << m) - 1;
    for (uint32_t t = 0; t < nterms; t++) {
        const lgpu_bterm_t tm = terms[t];
        double re = 0.0, im = 0.0;
        for (int e = threadIdx.x; e < E; e += blockDim.x) {
            const int f = e ^ int(tm.tflip);
            const uint64_t gf = base + hi_off[f >> m] + uint64_t(f & lowmask);
            const double sg = (__popcll(gf & tm.sign) & 1) ? -1.0 : 1.0;
            const cplx_t<T> a = tile[e], b = tile[f];
            re += sg * (double(a.x) * b.x + double(a.y) * b.y);
            im += sg * (double(a.x) * b.y - double(a.y) * b.x);
        }
        acc += tm.cr * re - tm.ci * im;
    }
    return acc;
}

__device__ __forceinline__ double block_sum(double v, double *red) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __syncthreads();
    if (lane == 0) red[warp] = v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0)
        for (int w = 0; w < int(blockDim.x >> 5); w++) s += red[w];  // fixed order
    return s;  // valid in thread 0
}

// --- bulk-copy helpers (TMA engine), bounded waits ---------------------------
__device__ unsigned int g_batch_error = 0;
constexpr int kRing = 3;
constexpr uint32_t kBatchWaitLimit = 1u << 24;

__device__ __forceinline__ uint32_t b_smem(const void *p) { return static_cast<uint32_t>(__cvta_generic_to_shared(p)); }
__device__ __forceinline__ void b_mbar_init(uint64_t *bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(b_smem(bar)) : "memory");
}
__device__ __forceinline__ void b_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(b_smem(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool b_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(b_smem(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ void b_load(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     b_smem(dst)),
                 "l"(src), "r"(bytes), "r"(b_smem(bar))
                 : "memory");
}
__device__ __forceinline__ void b_store(void *dst, const void *src, uint32_t bytes) {
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst), "r"(b_smem(src)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void b_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
__device__ __forceinline__ void b_wait_read_2() { asm volatile("cp.async.bulk.wait_group.read 2;" ::: "memory"); }
__device__ __forceinline__ void b_wait_read_1() { asm volatile("cp.async.bulk.wait_group.read 1;" ::: "memory"); }
__device__ __forceinline__ void b_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }
__device__ __forceinline__ void b_fence() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// DFM (complex128): gates run in float-float on a float-float tile.  A
// circuit's state is float-float from its first block (|0...0> is built in
// that form) to its last, in shared memory or in the CTA's scratch between
// blocks; only the last block converts its tiles to complex128, for the
// observable.
template <class T, bool EMU, bool DFM = false>
__global__ void __launch_bounds__(512, 1) batch_kernel(lgpu_batch_args_t a, unsigned *err) {
    using C = cplx_t<T>;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    C *ring = reinterpret_cast<C *>(smem_raw);
    __shared__ uint64_t hi_off[64];
    __shared__ double red[32];
    __shared__ uint32_t s_idx;
    __shared__ __align__(8) uint64_t full_bar[kRing];
    __shared__ uint32_t s_lm[kObsTermsCached];  // observable terms of the current last block
    __shared__ C s_c[kObsTermsCached];
    C *scratch = reinterpret_cast<C *>(a.scratch) + uint64_t(blockIdx.x) * a.scratch_amps;
    const uint32_t tile_amps = 1u << a.klarge;  // ring stage size (large circuits)
    if (threadIdx.x == 0) {
        for (int s = 0; s < kRing; s++) b_mbar_init(&full_bar[s]);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    uint64_t u = 0;            // running count of ring uses by this CTA (stage rotation)
    uint32_t phase_bits = 0;   // bit s: parity of the next completion of full_bar[s]
    bool failed = false;
    for (;;) {
        if (threadIdx.x == 0) s_idx = atomicAdd(a.counter, 1u);
        __syncthreads();
        const uint32_t ci = s_idx;
        __syncthreads();
        if (ci >= a.ncircuits || failed) break;
        const lgpu_bcircuit_t cir = a.circuits[a.order ? a.order[ci] : ci];
        double acc = 0.0;
        for (uint32_t bi = 0; bi < cir.block_cnt && !failed; bi++) {
            const lgpu_bblock_t blk = a.blocks[cir.block_off + bi];
            const int k = blk.k, mlow = blk.m;
            const int E = 1 << k;
            const bool first = bi == 0, last = bi + 1 == cir.block_cnt;
            if (threadIdx.x < 64) {
                uint64_t o = 0;
                for (int q = mlow; q < k; q++)
                    if ((threadIdx.x >> (q - mlow)) & 1) o |= uint64_t(1) << blk.bits[q];
                hi_off[threadIdx.x] = o;
            }
            const bool wht = last && k >= 3 && cir.obs_cnt <= kObsTermsCached;
            if (wht) {
                for (uint32_t t = threadIdx.x; t < cir.obs_cnt; t += blockDim.x) {
                    const lgpu_bterm_t tm = a.terms[cir.obs_off + t];
                    uint32_t L = 0;
                    for (int q = 0; q < k; q++)
                        if ((tm.sign >> blk.bits[q]) & 1u) L |= 1u << q;
                    s_lm[t] = L | (uint32_t(__popc(uint32_t(tm.tflip) & L) & 1) << 31);
                    s_c[t] = mk<T>(T(tm.cr), T(tm.ci));
                }
            }
            __syncthreads();
            auto tile_base = [&](uint64_t tau) {
                uint64_t base = tau;
                for (int q = 0; q < k; q++) {
                    const uint64_t lo = (uint64_t(1) << blk.bits[q]) - 1;
                    base = ((base & ~lo) << 1) | (base & lo);
                }
                return base;
            };
            if (k == int(cir.n)) {
                // ---- whole state in shared memory ----
                C *tile = ring;
                if constexpr (DFM) {  // |0...0> in float-float form: (1, 0, 0, 0) and zeros
                    for (int e = threadIdx.x; e < E; e += blockDim.x)
                        reinterpret_cast<float4 *>(tile)[e] = make_float4(e == 0 ? 1.0f : 0.0f, 0.0f, 0.0f, 0.0f);
                } else {
                    for (int e = threadIdx.x; e < E; e += blockDim.x) tile[e] = mk<T>(T(e == 0 ? 1 : 0), T(0));
                }
                __syncthreads();
                for (uint32_t gi = 0; gi < blk.gate_cnt; gi++) {
                    const lgpu_bgate_t g = a.gates[blk.gate_off + gi];
                    if (g.kind == BK_CHAINED) continue;
                    if constexpr (DFM)
                        tile_gate_df(reinterpret_cast<float4 *>(tile), E, g, a.pool);
                    else
                        tile_gate<T, EMU>(tile, E, g, a.pool);
                    __syncthreads();
                }
                if constexpr (DFM) {
                    tile_from_df(tile, E);
                    __syncthreads();
                }
                acc += wht ? tile_obs<T>(tile, k, a.terms + cir.obs_off, cir.obs_cnt, 0, s_lm, s_c)
                           : tile_obs_direct<T>(tile, E, a.terms + cir.obs_off, cir.obs_cnt, 0, mlow, hi_off);
                __syncthreads();
                continue;
            }
            // ---- streamed tiles through the ring (bulk copies) ----
            const uint64_t ntiles = uint64_t(1) << (cir.n - uint32_t(k));
            const uint32_t seg_amps = 1u << mlow, nseg = 1u << (k - mlow);
            const uint32_t seg_bytes = seg_amps * uint32_t(sizeof(C));
            auto stage_ptr = [&](uint64_t use) { return ring + size_t(use % kRing) * tile_amps; };
            auto issue_load = [&](uint64_t tau, uint64_t use) {
                C *buf = stage_ptr(use);
                uint64_t *bar = &full_bar[use % kRing];
                const uint64_t base = tile_base(tau);
                b_expect_tx(bar, nseg * seg_bytes);
                for (uint32_t sg = 0; sg < nseg; sg++) b_load(buf + sg * seg_amps, scratch + base + hi_off[sg], seg_bytes, bar);
            };
            const uint64_t u0 = u;
            if (!first && threadIdx.x == 0)
                for (uint64_t j = 0; j < ntiles && j < uint64_t(kRing); j++) issue_load(j, u0 + j);
            for (uint64_t j = 0; j < ntiles; j++) {
                const uint64_t use = u0 + j;
                C *tile = stage_ptr(use);
                const uint64_t base = tile_base(j);
                if (first) {
                    // |0...0> needs no load: wait until the stage's previous store has read it
                    if (threadIdx.x == 0) b_wait_read_2();
                    __syncthreads();
                    for (int e = threadIdx.x; e < E; e += blockDim.x) tile[e] = mk<T>(T(0), T(0));  // zero in either form
                    __syncthreads();
                    if (threadIdx.x == 0 && base == 0) {
                        if constexpr (DFM)
                            reinterpret_cast<float4 *>(tile)[0] = make_float4(1.0f, 0.0f, 0.0f, 0.0f);
                        else
                            tile[0] = mk<T>(T(1), T(0));
                    }
                    __syncthreads();
                } else {
                    const int st = int(use % kRing);
                    const uint32_t parity = (phase_bits >> st) & 1u;
                    uint32_t spins = 0;
                    bool timed_out = false;
                    while (!b_try_wait(&full_bar[st], parity)) {
                        if (++spins > kBatchWaitLimit) {
                            timed_out = true;
                            break;
                        }
                    }
                    if (__syncthreads_or(timed_out)) {
                        if (threadIdx.x == 0) {
                            atomicOr(&g_batch_error, 1u);
                            atomicOr(err, 1u);
                            // the loads issued so far (tiles j .. kRing - 1 at j = 0,
                            // else j .. j + kRing - 2; one per stage) may still be
                            // landing in this CTA's shared memory: wait for them,
                            // bounded again, before the CTA leaves
                            const uint64_t last = j == 0 ? uint64_t(kRing - 1) : j + uint64_t(kRing) - 2;
                            for (uint64_t jj = j; jj <= last && jj < ntiles; jj++) {
                                const int s2 = int((u0 + jj) % kRing);
                                const uint32_t par2 = (phase_bits >> s2) & 1u;
                                for (uint32_t sp = 0; !b_try_wait(&full_bar[s2], par2) && sp <= kBatchWaitLimit; sp++) {
                                }
                            }
                        }
                        failed = true;
                        break;
                    }
                    phase_bits ^= 1u << st;
                }
                // float-float (DFM): the circuit's state stays in float-float form in
                // the scratch from block to block; only the last block converts back
                for (uint32_t gi = 0; gi < blk.gate_cnt; gi++) {
                    const lgpu_bgate_t g = a.gates[blk.gate_off + gi];
                    if (g.kind == BK_CHAINED || (base & g.omask) != g.oval) continue;  // tile-uniform
                    if constexpr (DFM)
                        tile_gate_df(reinterpret_cast<float4 *>(tile), E, g, a.pool);
                    else
                        tile_gate<T, EMU>(tile, E, g, a.pool);
                    __syncthreads();
                }
                if constexpr (DFM) {
                    if (last) {
                        tile_from_df(tile, E);
                        __syncthreads();
                    }
                }
                if (last) {
                    acc += wht ? tile_obs<T>(tile, k, a.terms + cir.obs_off, cir.obs_cnt, base, s_lm, s_c)
                               : tile_obs_direct<T>(tile, E, a.terms + cir.obs_off, cir.obs_cnt, base, mlow, hi_off);
                    __syncthreads();
                } else {
                    b_fence();
                    __syncthreads();
                    if (threadIdx.x == 0) {
                        for (uint32_t sg = 0; sg < nseg; sg++)
                            b_store(scratch + base + hi_off[sg], tile + sg * seg_amps, seg_bytes);
                        b_commit();
                    }
                }
                if (!first && threadIdx.x == 0 && j >= 1) {
                    // refill the previous stage once its store has finished reading it
                    const uint64_t next = (j - 1) + kRing;
                    if (next < ntiles) {
                        if (!last) b_wait_read_1();
                        issue_load(next, u0 + next);
                    }
                }
            }
            // (every load issued above is for a tile index < ntiles and is consumed)
            u = u0 + ntiles;
            // all stores of this block complete before the next block reads
            if (threadIdx.x == 0) b_wait_all();
            __threadfence();
            __syncthreads();
        }
        if (failed) break;
        const double total = block_sum(acc, red);
        if (threadIdx.x == 0) a.out[cir.out] = total;
        __syncthreads();
    }
    if (threadIdx.x == 0) b_wait_all();
}

lgpu_status_t batch_error_fetch(unsigned *v, bool reset) {
    LGPU_CUDA_TRY(cudaMemcpyFromSymbol(v, g_batch_error, sizeof(unsigned)));
    if (reset && *v) {
        unsigned z = 0;
        LGPU_CUDA_TRY(cudaMemcpyToSymbol(g_batch_error, &z, sizeof(z)));
    }
    return LGPU_OK;
}

template <class T, bool EMU, bool DFM = false>
static lgpu_status_t launch_batch(const lgpu_batch_args_t &args, unsigned grid, size_t smem, cudaStream_t s) {
    // The attribute is set once per size outside any stream capture (the host
    // runs the batch eagerly once before capturing it).
    static std::atomic<size_t> attr[64];
    LGPU_TRY(ensure_smem(reinterpret_cast<const void *>(batch_kernel<T, EMU, DFM>), smem, attr));
    unsigned *err = nullptr;
    LGPU_TRY(stream_error_ptr(s, &err));
    batch_kernel<T, EMU, DFM><<<grid, args.threads, smem, s>>>(args, err);
    LGPU_CHECK_LAUNCH();
    return LGPU_OK;
}

}  // namespace lgpu

using namespace lgpu;

extern "C" {

lgpu_status_t lgpu_batch_prepare(const lgpu_bgate_t *gates, uint64_t ngates, const double *params, double *pool,
                                 lgpu_dtype_t dt, lgpu_stream_t stream) {
    if (ngates == 0) return LGPU_OK;
    if (!gates || !pool) return fail(LGPU_ERR_INVALID_ARG, "null gates/pool");
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    if (dt != LGPU_C64 && dt != LGPU_C128) return fail(LGPU_ERR_INVALID_ARG, "unknown dtype");
    const int mode = dt == LGPU_C64 ? 1 : (batch_df() ? 2 : 0);
    bprep_kernel<<<grid_for(ngates, 128, 1, 4), 128, 0, s>>>(gates, ngates, params, pool, mode);
    LGPU_CHECK_LAUNCH();
    return LGPU_OK;
}

lgpu_status_t lgpu_batch_run(const lgpu_batch_args_t *args, lgpu_dtype_t dt, unsigned grid, lgpu_stream_t stream) {
    if (!args || !args->counter || !args->circuits || !args->out)
        return fail(LGPU_ERR_INVALID_ARG, "batch: null argument");
    if (args->kmax < 1 || args->kmax > (dt == LGPU_C128 ? 13u : 14u))
        return fail(LGPU_ERR_INVALID_ARG, "batch: tile size out of range");
    if (args->klarge < 6 || args->klarge > (dt == LGPU_C128 ? 12u : 13u))
        return fail(LGPU_ERR_INVALID_ARG, "batch: large-circuit tile size out of range");
    if (args->threads != 128 && args->threads != 256 && args->threads != 512)
        return fail(LGPU_ERR_INVALID_ARG, "batch: threads must be 128, 256 or 512");
    if (grid == 0) return fail(LGPU_ERR_INVALID_ARG, "batch: empty grid");
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const size_t amp = dt == LGPU_C128 ? 16 : 8;
    const size_t smem = std::max((size_t(1) << args->kmax) * amp, size_t(kRing) * (size_t(1) << args->klarge) * amp);
    if (dt == LGPU_C128)
        return batch_df()          ? launch_batch<double, false, true>(*args, grid, smem, s)
               : f64_mode() == 1 ? launch_batch<double, true>(*args, grid, smem, s)
                                 : launch_batch<double, false>(*args, grid, smem, s);
    return launch_batch<float, false>(*args, grid, smem, s);
}

}  // extern "C"
