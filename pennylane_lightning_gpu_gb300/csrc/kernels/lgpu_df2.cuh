// Paired float-float arithmetic: two lanes of float-float values held in
// 64-bit register pairs and computed with the paired FP32 instructions of the
// sm_100 family (mul / fma / add / sub .rn.f32x2).  Each lane performs exactly
// the operations of the scalar float-float code in lgpu_df64.cuh, in the same
// order and with the same rounding, so results are bit-identical to it.  A
// paired instruction takes one issue slot for two FP32 operations (the FMA
// pipe still spends two cycles on it), which relieves kernels that are bound
// by instruction issue rather than by the FMA pipe.
//
// Used by the complex128 fused gate blocks with lanes (re, im) of one
// amplitude: the tile holds (re.hi, im.hi, re.lo, im.lo) per amplitude, so a
// float4 load gives the lane pairs (re.hi, im.hi) and (re.lo, im.lo) directly.
#pragma once

#include "lgpu_df64.cuh"

namespace lgpu {

struct F2 {
    unsigned long long v;
};

__device__ __forceinline__ F2 f2_pack(float a, float b) {
    F2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r.v) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ float f2_x(F2 a) { return __uint_as_float(static_cast<unsigned>(a.v)); }
__device__ __forceinline__ float f2_y(F2 a) { return __uint_as_float(static_cast<unsigned>(a.v >> 32)); }
__device__ __forceinline__ F2 f2_mul(F2 a, F2 b) {
    F2 r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
    return r;
}
__device__ __forceinline__ F2 f2_fma(F2 a, F2 b, F2 c) {
    F2 r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r.v) : "l"(a.v), "l"(b.v), "l"(c.v));
    return r;
}
__device__ __forceinline__ F2 f2_add(F2 a, F2 b) {
    F2 r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
    return r;
}
__device__ __forceinline__ F2 f2_sub(F2 a, F2 b) {
    F2 r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
    return r;
}

// Lane k holds the float-float value (hi.k, lo.k).
struct DF2 {
    F2 hi, lo;
};

// Lanes (a, b) from two float-float scalars.
__device__ __forceinline__ DF2 df2_of(DF a, DF b) { return DF2{f2_pack(a.hi, b.hi), f2_pack(a.lo, b.lo)}; }

// m * x per lane, unnormalised, as df_mul: hi = fl(m.hi x.hi), lo = its exact
// error (a scalar FMA per lane, which negates an operand for free) plus
// m.lo x.hi, then plus m.hi x.lo.
__device__ __forceinline__ DF2 df2_mul(const DF2 &m, const DF2 &x) {
    const F2 p = f2_mul(m.hi, x.hi);
    const float ex = __fmaf_rn(f2_x(m.hi), f2_x(x.hi), -f2_x(p));
    const float ey = __fmaf_rn(f2_y(m.hi), f2_y(x.hi), -f2_y(p));
    F2 e = f2_fma(m.lo, x.hi, f2_pack(ex, ey));
    e = f2_fma(m.hi, x.lo, e);
    return DF2{p, e};
}

// The sum of K unnormalised pairs per lane, as df_sum.
template <int K> __device__ __forceinline__ DF2 df2_sum(const DF2 (&t)[K]) {
    F2 s = t[0].hi, c = t[0].lo;
#pragma unroll
    for (int k = 1; k < K; k++) {
        const F2 a = s, b = t[k].hi;
        s = f2_add(a, b);
        const F2 bb = f2_sub(s, a);
        const F2 err = f2_add(f2_sub(a, f2_sub(s, bb)), f2_sub(b, bb));
        c = f2_add(c, f2_add(err, t[k].lo));
    }
    const F2 h = f2_add(s, c);
    return DF2{h, f2_sub(c, f2_sub(h, s))};
}

// The coefficient lanes of a 2x2 given as body1_dfv's m (8 float-float
// values, (re, im) interleaved, row-major): c[i] = (m_i, m_i) for the real
// parts (even i) and (-m_i, m_i) for the imaginary parts (odd i), because
// (m.re + i m.im) x = m.re (xr, xi) + (-m.im, m.im) (xi, xr).
__device__ __forceinline__ void df2_coeffs(const DF *m, DF2 (&c)[8]) {
#pragma unroll
    for (int i = 0; i < 8; i++) c[i] = df2_of((i & 1) ? df_neg(m[i]) : m[i], m[i]);
}

// The structured 2x2 bodies of body1_dfv on amplitudes x, y held as lanes
// (re, im), with the coefficient lanes of df2_coeffs.  xs / ys are x / y
// with the lanes swapped, (im, re), for the imaginary-part products.  Each
// output lane sums the same terms in the same order as the scalar body.
template <int BODY> __device__ __forceinline__ void body1_df2(const DF2 (&c)[8], DF2 &x, DF2 &y) {
    const DF2 xs{f2_pack(f2_y(x.hi), f2_x(x.hi)), f2_pack(f2_y(x.lo), f2_x(x.lo))};
    const DF2 ys{f2_pack(f2_y(y.hi), f2_x(y.hi)), f2_pack(f2_y(y.lo), f2_x(y.lo))};
    DF2 o0, o1;
    if constexpr (BODY == 1) {  // diagonal
        o0 = df2_sum<2>({df2_mul(c[0], x), df2_mul(c[1], xs)});
        o1 = df2_sum<2>({df2_mul(c[6], y), df2_mul(c[7], ys)});
    } else if constexpr (BODY == 3) {  // antidiagonal
        o0 = df2_sum<2>({df2_mul(c[2], y), df2_mul(c[3], ys)});
        o1 = df2_sum<2>({df2_mul(c[4], x), df2_mul(c[5], xs)});
    } else if constexpr (BODY == 4) {  // real
        o0 = df2_sum<2>({df2_mul(c[0], x), df2_mul(c[2], y)});
        o1 = df2_sum<2>({df2_mul(c[4], x), df2_mul(c[6], y)});
    } else if constexpr (BODY == 5) {  // RX-like
        o0 = df2_sum<2>({df2_mul(c[0], x), df2_mul(c[3], ys)});
        o1 = df2_sum<2>({df2_mul(c[0], y), df2_mul(c[5], xs)});
    } else {  // dense
        o0 = df2_sum<4>({df2_mul(c[0], x), df2_mul(c[1], xs), df2_mul(c[2], y), df2_mul(c[3], ys)});
        o1 = df2_sum<4>({df2_mul(c[4], x), df2_mul(c[5], xs), df2_mul(c[6], y), df2_mul(c[7], ys)});
    }
    x = o0;
    y = o1;
}

}  // namespace lgpu
