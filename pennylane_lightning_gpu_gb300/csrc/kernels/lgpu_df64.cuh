// Float-float ("df64") arithmetic for complex128 gate bodies on GB300.
//
// GB300 issues about 2 FP64 operations per clock per SM against about 128
// FP32 ones, and conversions between double and float run on the FP64 pipe
// too.  A complex128 gate body can instead carry each double as an unevaluated
// sum hi + lo of two floats (about 48 significant bits): products by the
// exact TwoProd of an FMA, sums by Knuth's TwoSum, all on the FP32 pipe.  The
// state stays complex128 in memory; the split of a double into hi + lo and
// the rebuild of the double are integer bit operations, so a body issues no
// FP64 instruction at all.
//
//   df_from_double(d): hi = d with its mantissa truncated to 24 bits, lo = the
//     remaining 29 bits truncated to 24; |d - (hi + lo)| < 2^-47 |d| + 2^-126
//     (lo leaves the float range below |d| = 2^-102 and is then dropped;
//     |d| < 2^-126 gives 0: such amplitudes are below any tolerance).  Inf and
//     NaN give hi = Inf / NaN.
//   df_to_double(x): the double nearest below |hi + lo| (truncation: at most
//     one ulp of the double), exact when hi + lo fits 53 bits, as it does for
//     a normalised pair.
//   df_sum: TwoSum over the high parts, the low parts and the rounding errors
//     added in float, then renormalised (Fast2Sum): error about 2^-47 of the
//     largest term.
//
// Every product and sum goes through __fmul_rn / __fadd_rn on the device so
// that the compiler cannot contract them into FMAs (which would break the
// exact-error identities).  The host versions let the arithmetic be
// unit-tested with a plain C++ compiler.
#pragma once

#include <stdint.h>

#include <cmath>
#include <cstring>

#include "lgpu_f64emu.cuh"

namespace lgpu {

struct DF {
    float hi, lo;
};

LGPU_HD uint32_t df_fbits(float x) {
#if defined(__CUDA_ARCH__)
    return __float_as_uint(x);
#else
    uint32_t b;
    std::memcpy(&b, &x, sizeof(b));
    return b;
#endif
}
LGPU_HD float df_ffrom(uint32_t b) {
#if defined(__CUDA_ARCH__)
    return __uint_as_float(b);
#else
    float x;
    std::memcpy(&x, &b, sizeof(x));
    return x;
#endif
}
LGPU_HD int df_clz32(uint32_t x) {
#if defined(__CUDA_ARCH__)
    return __clz(x);
#else
    return x ? __builtin_clz(x) : 32;
#endif
}
LGPU_HD int df_clz64(uint64_t x) {
#if defined(__CUDA_ARCH__)
    return __clzll(static_cast<long long>(x));
#else
    return x ? __builtin_clzll(x) : 64;
#endif
}
LGPU_HD float df_mul_rn(float a, float b) {
#if defined(__CUDA_ARCH__)
    return __fmul_rn(a, b);
#else
    return a * b;
#endif
}
LGPU_HD float df_add_rn(float a, float b) {
#if defined(__CUDA_ARCH__)
    return __fadd_rn(a, b);
#else
    return a + b;
#endif
}
LGPU_HD float df_sub_rn(float a, float b) {
#if defined(__CUDA_ARCH__)
    return __fsub_rn(a, b);
#else
    return a - b;
#endif
}
LGPU_HD float df_fma(float a, float b, float c) {
#if defined(__CUDA_ARCH__)
    return __fmaf_rn(a, b, c);
#else
    return std::fmaf(a, b, c);
#endif
}

// Split of a double constant on the host (round to nearest, then the
// remainder): |d - (hi + lo)| <= 2^-48 |d|.
inline DF df_split_host(double d) {
    DF r;
    r.hi = static_cast<float>(d);
    r.lo = static_cast<float>(d - static_cast<double>(r.hi));
    return r;
}

LGPU_HD DF df_from_double(double d) {
    const uint64_t b = emu_bits(d);
    const uint32_t sign = uint32_t(b >> 32) & 0x80000000u;
    const int e = int((b >> 52) & 0x7FFu);
    const uint64_t mant = b & ((uint64_t(1) << 52) - 1u);
    DF r;
    if (e == 0x7FF) {  // Inf / NaN
        r.hi = df_ffrom(sign | 0x7F800000u | (mant ? 0x400000u : 0u));
        r.lo = 0.0f;
        return r;
    }
    const int ef = e - 1023 + 127;  // float biased exponent of hi
    if (ef <= 0) {                  // |d| < 2^-126, zero and subnormals
        r.hi = df_ffrom(sign);
        r.lo = df_ffrom(sign);
        return r;
    }
    if (ef >= 255) {  // |d| >= 2^128: beyond every amplitude and coefficient
        r.hi = df_ffrom(sign | 0x7F800000u);
        r.lo = 0.0f;
        return r;
    }
    r.hi = df_ffrom(sign | (uint32_t(ef) << 23) | uint32_t(mant >> 29));
    const uint32_t low = uint32_t(mant & 0x1FFFFFFFu);  // value low * 2^(e - 1075)
    if (low == 0) {
        r.lo = df_ffrom(sign);
        return r;
    }
    const int lz = df_clz32(low) - 3;  // the top bit of low << lz is bit 28
    const int el = ef - 24 - lz;       // float biased exponent of lo
    r.lo = el > 0 ? df_ffrom(sign | (uint32_t(el) << 23) | (((low << lz) >> 5) & 0x7FFFFFu)) : df_ffrom(sign);
    return r;
}

LGPU_HD double df_to_double(DF x) {
    const uint32_t hb = df_fbits(x.hi), lb = df_fbits(x.lo);
    const int he = int((hb >> 23) & 0xFFu), le = int((lb >> 23) & 0xFFu);
    if (he == 0xFF)  // Inf / NaN: keep the class (a NaN keeps a quiet bit)
        return emu_double((uint64_t(hb >> 31) << 63) | (uint64_t(0x7FF) << 52) | (uint64_t(hb & 0x7FFFFFu) << 29));
    if (he == 0 && le == 0) return emu_double(uint64_t(hb >> 31) << 63);  // (subnormal floats flush)
    // Integers in units of 2^(E - 1075 + 896) where E = the exponent of the
    // larger part: H = 24-bit significand << 29, L aligned to it.
    const int eref = he >= le ? he : le;
    int64_t H = 0, L = 0;
    if (he != 0) {
        const int s = he - eref + 29;
        const uint64_t m = uint64_t((hb & 0x7FFFFFu) | 0x800000u);
        H = int64_t(s >= 0 ? (m << s) : (s > -24 ? (m >> -s) : 0u));
        if (hb >> 31) H = -H;
    }
    if (le != 0) {
        const int s = le - eref + 29;
        const uint64_t m = uint64_t((lb & 0x7FFFFFu) | 0x800000u);
        L = int64_t(s >= 0 ? (m << s) : (s > -24 ? (m >> -s) : 0u));
        if (lb >> 31) L = -L;
    }
    const int64_t S = H + L;
    if (S == 0) return emu_double(uint64_t(hb >> 31) << 63);
    const uint64_t neg = S < 0 ? 1u : 0u;
    const uint64_t A = uint64_t(S < 0 ? -S : S);  // < 2^54
    const int p = 63 - df_clz64(A);               // top bit
    const uint64_t M = p >= 52 ? (A >> (p - 52)) : (A << (52 - p));
    const int E = p + eref + 844;  // biased exponent of the double: 2^(p + eref - 127 - 52)
    return emu_double((neg << 63) | (uint64_t(E) << 52) | (M & ((uint64_t(1) << 52) - 1u)));
}

// m * x, unnormalised: hi = fl(m.hi x.hi), lo = its exact error plus the
// cross terms (m.lo x.lo, below 2^-48, is dropped).
LGPU_HD DF df_mul(DF m, DF x) {
    const float p = df_mul_rn(m.hi, x.hi);
    float e = df_fma(m.hi, x.hi, -p);
    e = df_fma(m.hi, x.lo, df_fma(m.lo, x.hi, e));
    return DF{p, e};
}

template <int K> LGPU_HD DF df_sum(const DF (&t)[K]) {
    float s = t[0].hi, c = t[0].lo;
#pragma unroll
    for (int k = 1; k < K; k++) {
        const float a = s, b = t[k].hi;
        s = df_add_rn(a, b);
        const float bb = df_sub_rn(s, a);
        const float err = df_add_rn(df_sub_rn(a, df_sub_rn(s, bb)), df_sub_rn(b, bb));
        c = df_add_rn(c, df_add_rn(err, t[k].lo));
    }
    const float h = df_add_rn(s, c);
    return DF{h, df_sub_rn(c, df_sub_rn(h, s))};
}

LGPU_HD DF df_neg(DF x) { return DF{-x.hi, -x.lo}; }

// conj(a) . (M a) over one group of D amplitudes, added to (re, im).  m holds
// M row-major as (re, im) float-float pairs; a = ar + i ai.  Each row
// x_r = sum_c M_rc a_c is formed in float-float, then re += Re(conj(a_r) x_r)
// and im += Im(conj(a_r) x_r).  The row loop stays rolled (the columns are
// unrolled); a_r is picked from the arrays by compile-time selects, so the
// arrays stay in registers.
template <int D, class MAT>
LGPU_HD void df_expval_group(const MAT &m, const DF (&ar)[D], const DF (&ai)[D], DF &re, DF &im) {
#pragma unroll 1
    for (int r = 0; r < D; r++) {
        DF xr{0.0f, 0.0f}, xi{0.0f, 0.0f};
#pragma unroll
        for (int c = 0; c < D; c++) {
            const DF mr = m[2 * (r * D + c)], mi = m[2 * (r * D + c) + 1];
            xr = df_sum<3>({xr, df_mul(mr, ar[c]), df_neg(df_mul(mi, ai[c]))});
            xi = df_sum<3>({xi, df_mul(mr, ai[c]), df_mul(mi, ar[c])});
        }
        DF pr = ar[0], pi = ai[0];
#pragma unroll
        for (int k = 1; k < D; k++)
            if (k == r) {
                pr = ar[k];
                pi = ai[k];
            }
        re = df_sum<3>({re, df_mul(pr, xr), df_mul(pi, xi)});
        im = df_sum<3>({im, df_mul(pr, xi), df_neg(df_mul(pi, xr))});
    }
}

// Body code of a diagonal with entries exactly +1 or -1 (CZ, Z, their
// controlled forms): the float-float kernels flip signs instead of
// multiplying.  Only these kernels know the code; the host sets it.
constexpr int kDfSignDiag = 6;

// True for a 2x2 (re, im interleaved) that is diag(+-1, +-1).
inline bool df_sign_diag_host(const double *m) {
    auto pm1 = [](double v) { return v == 1.0 || v == -1.0; };
    return pm1(m[0]) && m[1] == 0.0 && m[2] == 0.0 && m[3] == 0.0 && m[4] == 0.0 && m[5] == 0.0 && pm1(m[6]) &&
           m[7] == 0.0;
}

// The structured 2x2 bodies (Body1 in lgpu_bodies.cuh) in float-float on
// float-float amplitudes x = (xr, xi), y = (yr, yi).  m holds the 8 real
// coefficients (re, im interleaved, row-major) as pairs.  Body codes: 0 dense,
// 1 diagonal, 2 permutation, 3 antidiagonal, 4 real, 5 RX-like (m00 = m11 = c
// real, m01 = i u, m10 = i v).
template <int BODY> LGPU_HD void body1_dfv(const DF *m, DF &xr, DF &xi, DF &yr, DF &yi) {
    if constexpr (BODY == kDfSignDiag) {  // diag(s0, s1), s = +-1 exactly: sign flips, no rounding
        const float s0 = m[0].hi, s1 = m[6].hi;
        xr = DF{xr.hi * s0, xr.lo * s0};
        xi = DF{xi.hi * s0, xi.lo * s0};
        yr = DF{yr.hi * s1, yr.lo * s1};
        yi = DF{yi.hi * s1, yi.lo * s1};
    } else if constexpr (BODY == 2) {
        const DF a = xr, b = xi;
        xr = yr;
        xi = yi;
        yr = a;
        yi = b;
    } else {
        DF r0, i0, r1, i1;
        if constexpr (BODY == 1) {
            r0 = df_sum<2>({df_mul(m[0], xr), df_mul(df_neg(m[1]), xi)});
            i0 = df_sum<2>({df_mul(m[0], xi), df_mul(m[1], xr)});
            r1 = df_sum<2>({df_mul(m[6], yr), df_mul(df_neg(m[7]), yi)});
            i1 = df_sum<2>({df_mul(m[6], yi), df_mul(m[7], yr)});
        } else if constexpr (BODY == 3) {
            r0 = df_sum<2>({df_mul(m[2], yr), df_mul(df_neg(m[3]), yi)});
            i0 = df_sum<2>({df_mul(m[2], yi), df_mul(m[3], yr)});
            r1 = df_sum<2>({df_mul(m[4], xr), df_mul(df_neg(m[5]), xi)});
            i1 = df_sum<2>({df_mul(m[4], xi), df_mul(m[5], xr)});
        } else if constexpr (BODY == 4) {
            r0 = df_sum<2>({df_mul(m[0], xr), df_mul(m[2], yr)});
            i0 = df_sum<2>({df_mul(m[0], xi), df_mul(m[2], yi)});
            r1 = df_sum<2>({df_mul(m[4], xr), df_mul(m[6], yr)});
            i1 = df_sum<2>({df_mul(m[4], xi), df_mul(m[6], yi)});
        } else if constexpr (BODY == 5) {
            r0 = df_sum<2>({df_mul(m[0], xr), df_mul(df_neg(m[3]), yi)});
            i0 = df_sum<2>({df_mul(m[0], xi), df_mul(m[3], yr)});
            r1 = df_sum<2>({df_mul(m[0], yr), df_mul(df_neg(m[5]), xi)});
            i1 = df_sum<2>({df_mul(m[0], yi), df_mul(m[5], xr)});
        } else {
            r0 = df_sum<4>({df_mul(m[0], xr), df_mul(df_neg(m[1]), xi), df_mul(m[2], yr), df_mul(df_neg(m[3]), yi)});
            i0 = df_sum<4>({df_mul(m[0], xi), df_mul(m[1], xr), df_mul(m[2], yi), df_mul(m[3], yr)});
            r1 = df_sum<4>({df_mul(m[4], xr), df_mul(df_neg(m[5]), xi), df_mul(m[6], yr), df_mul(df_neg(m[7]), yi)});
            i1 = df_sum<4>({df_mul(m[4], xi), df_mul(m[5], xr), df_mul(m[6], yi), df_mul(m[7], yr)});
        }
        xr = r0;
        xi = i0;
        yr = r1;
        yi = i1;
    }
}

// The same on complex128 values: split, apply, rebuild.
template <int BODY> LGPU_HD void body1_df(const DF *m, double &x_re, double &x_im, double &y_re, double &y_im) {
    DF xr = df_from_double(x_re), xi = df_from_double(x_im);
    DF yr = df_from_double(y_re), yi = df_from_double(y_im);
    body1_dfv<BODY>(m, xr, xi, yr, yi);
    x_re = df_to_double(xr);
    x_im = df_to_double(xi);
    y_re = df_to_double(yr);
    y_im = df_to_double(yi);
}

}  // namespace lgpu
