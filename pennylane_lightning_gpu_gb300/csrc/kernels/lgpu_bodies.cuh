// 1-target gate bodies shared by the gate, fused and batched kernels, and the
// index expansion that enumerates a gate's amplitude pairs inside a
// shared-memory tile.
#pragma once

#include "lgpu_f64emu.cuh"
#include "lgpu_internal.cuh"

namespace lgpu {

enum Body1 : int { B_DENSE = 0, B_DIAG = 1, B_PERM = 2, B_ANTIDIAG = 3, B_REAL = 4, B_RXLIKE = 5 };

template <class T, class I> struct G1Params {
    Holes holes;
    I tbit;
    I cset;
    I ngroups;
    T m[8];
    KConst k[4];  // integer-pipe multipliers (complex128 EMU bodies)
};

template <class T, int BODY>
__device__ __forceinline__ void body1(const T *m, cplx_t<T> &a0, cplx_t<T> &a1) {
    using C = cplx_t<T>;
    const C x = a0, y = a1;
    if constexpr (BODY == B_PERM) {
        a0 = y;
        a1 = x;
    } else if constexpr (BODY == B_DIAG) {
        a0 = mk<T>(fmaT(m[0], x.x, -m[1] * x.y), fmaT(m[0], x.y, m[1] * x.x));
        a1 = mk<T>(fmaT(m[6], y.x, -m[7] * y.y), fmaT(m[6], y.y, m[7] * y.x));
    } else if constexpr (BODY == B_ANTIDIAG) {
        a0 = mk<T>(fmaT(m[2], y.x, -m[3] * y.y), fmaT(m[2], y.y, m[3] * y.x));
        a1 = mk<T>(fmaT(m[4], x.x, -m[5] * x.y), fmaT(m[4], x.y, m[5] * x.x));
    } else if constexpr (BODY == B_REAL) {
        a0 = mk<T>(fmaT(m[0], x.x, m[2] * y.x), fmaT(m[0], x.y, m[2] * y.y));
        a1 = mk<T>(fmaT(m[4], x.x, m[6] * y.x), fmaT(m[4], x.y, m[6] * y.y));
    } else if constexpr (BODY == B_RXLIKE) {
        // m00 = m11 = c (real), m01 = i*u, m10 = i*v (u, v real)
        const T c = m[0], u = m[3], v = m[5];
        a0 = mk<T>(fmaT(c, x.x, -u * y.y), fmaT(c, x.y, u * y.x));
        a1 = mk<T>(fmaT(c, y.x, -v * x.y), fmaT(c, y.y, v * x.x));
    } else {
        C r0 = mk<T>(m[0] * x.x, m[0] * x.y);
        r0.x = fmaT(-m[1], x.y, r0.x);
        r0.y = fmaT(m[1], x.x, r0.y);
        r0.x = fmaT(m[2], y.x, r0.x);
        r0.y = fmaT(m[2], y.y, r0.y);
        r0.x = fmaT(-m[3], y.y, r0.x);
        r0.y = fmaT(m[3], y.x, r0.y);
        C r1 = mk<T>(m[4] * x.x, m[4] * x.y);
        r1.x = fmaT(-m[5], x.y, r1.x);
        r1.y = fmaT(m[5], x.x, r1.y);
        r1.x = fmaT(m[6], y.x, r1.x);
        r1.y = fmaT(m[6], y.y, r1.y);
        r1.x = fmaT(-m[7], y.y, r1.x);
        r1.y = fmaT(m[7], y.x, r1.y);
        a0 = r0;
        a1 = r1;
    }
}

// complex128 bodies with one DFMA + one integer-pipe multiply per output
// component (half the FP64 issue of body1).  k[] holds the constants the
// host prepared for the body (see run_gate1).
template <int BODY>
__device__ __forceinline__ void body1_emu(const double *m, const KConst *k, double2 &a0, double2 &a1) {
    const double2 x = a0, y = a1;
    if constexpr (BODY == B_PERM) {
        a0 = y;
        a1 = x;
    } else if constexpr (BODY == B_DIAG) {  // k = {-m00i, m00i, -m11i, m11i}
        a0 = make_double2(__fma_rn(m[0], x.x, emul(x.y, k[0])), __fma_rn(m[0], x.y, emul(x.x, k[1])));
        a1 = make_double2(__fma_rn(m[6], y.x, emul(y.y, k[2])), __fma_rn(m[6], y.y, emul(y.x, k[3])));
    } else if constexpr (BODY == B_ANTIDIAG) {  // k = {-m01i, m01i, -m10i, m10i}
        a0 = make_double2(__fma_rn(m[2], y.x, emul(y.y, k[0])), __fma_rn(m[2], y.y, emul(y.x, k[1])));
        a1 = make_double2(__fma_rn(m[4], x.x, emul(x.y, k[2])), __fma_rn(m[4], x.y, emul(x.x, k[3])));
    } else if constexpr (BODY == B_REAL) {  // k = {m01r, m10r}
        a0 = make_double2(__fma_rn(m[0], x.x, emul(y.x, k[0])), __fma_rn(m[0], x.y, emul(y.y, k[0])));
        a1 = make_double2(__fma_rn(m[6], y.x, emul(x.x, k[1])), __fma_rn(m[6], y.y, emul(x.y, k[1])));
    } else if constexpr (BODY == B_RXLIKE) {  // k = {-u, u, -v, v}
        const double c = m[0];
        a0 = make_double2(__fma_rn(c, x.x, emul(y.y, k[0])), __fma_rn(c, x.y, emul(y.x, k[1])));
        a1 = make_double2(__fma_rn(c, y.x, emul(x.y, k[2])), __fma_rn(c, y.y, emul(x.x, k[3])));
    } else {  // dense: k = {m00i, m01i, m10i, m11i}; 12 FP64 operations per pair instead of 16
        const double t0 = emul(x.y, k[0]) + emul(y.y, k[1]);
        const double t1 = emul(x.x, k[0]) + emul(y.x, k[1]);
        const double t2 = emul(x.y, k[2]) + emul(y.y, k[3]);
        const double t3 = emul(x.x, k[2]) + emul(y.x, k[3]);
        a0 = make_double2(__fma_rn(m[0], x.x, __fma_rn(m[2], y.x, -t0)), __fma_rn(m[0], x.y, __fma_rn(m[2], y.y, t1)));
        a1 = make_double2(__fma_rn(m[4], x.x, __fma_rn(m[6], y.x, -t2)), __fma_rn(m[4], x.y, __fma_rn(m[6], y.y, t3)));
    }
}

template <class T, int BODY, bool EMU>
__device__ __forceinline__ void body1_sel(const T *m, const KConst *k, cplx_t<T> &a0, cplx_t<T> &a1) {
    if constexpr (EMU && sizeof(T) == 8)
        body1_emu<BODY>(reinterpret_cast<const double *>(m), k, reinterpret_cast<double2 &>(a0),
                        reinterpret_cast<double2 &>(a1));
    else
        body1<T, BODY>(m, a0, a1);
}

// Enumeration of a gate's amplitude groups inside a shared-memory tile.
// `holes` marks the tile positions of the gate's targets and in-tile
// controls; the f-th group starts at f with zeros inserted at the holes (the
// control values are OR-ed in afterwards), so no lane idles on a control
// test.  A thread visits f = start, start + stride, ...: the starts differ by
// the stride with zeros inserted, and ((x | holes) + inc) & ~holes adds it
// with the carries running through the hole positions (three integer
// operations per group instead of one insertion per hole).
__device__ __forceinline__ uint32_t insert_zeros(uint32_t f, uint32_t holes) {
    for (uint32_t m = holes; m; m &= m - 1u) {
        const uint32_t low = (m & (0u - m)) - 1u;
        f = ((f & ~low) << 1) | (f & low);
    }
    return f;
}

struct PairWalk {
    uint32_t x, inc, holes;
    __device__ __forceinline__ PairWalk(uint32_t holes_, uint32_t start, uint32_t stride)
        : x(insert_zeros(start, holes_)), inc(insert_zeros(stride, holes_)), holes(holes_) {}
    __device__ __forceinline__ void step() { x = ((x | holes) + inc) & ~holes; }
};

// Shared-memory tiles are stored swizzled: the 16-byte chunk c of 128-byte
// row r lives at chunk c ^ (r mod 8) (complex64: element e -> e ^
// (((e >> 4) & 7) << 1); complex128: e -> e ^ ((e >> 3) & 7)).  A warp
// reading one element from each of 32 rows (a register group on the lowest
// tile positions) then spreads over the banks, 16-byte chunks stay whole
// (so 16-byte asynchronous copies can fill the layout), and accesses within
// a row are only permuted.
template <class T> __device__ __forceinline__ int swz(int e) {
    if constexpr (sizeof(T) == 4)
        return e ^ (((e >> 4) & 7) << 1);
    else
        return e ^ ((e >> 3) & 7);
}

// Register groups: a run of consecutive 1-target gates whose targets and
// in-tile controls lie on R tile positions is applied with each thread
// holding the 2^R amplitudes of one index group in registers (one
// shared-memory round trip and one barrier per group instead of per gate).
// A gate is given by its local target LT (0..R-1), the local control mask and
// values, its body and coefficients.
template <class T, int R, int LT, int BODY, bool EMU>
__device__ __forceinline__ void reg_gate(cplx_t<T> (&a)[1 << R], const T *m, const KConst *k, uint32_t lcm,
                                         uint32_t lcv) {
    T mr[8];
#pragma unroll
    for (int i = 0; i < 8; i++) mr[i] = m[i];
    KConst kr[4];
#pragma unroll
    for (int i = 0; i < 4; i++) kr[i] = EMU ? k[i] : KConst{};
#pragma unroll
    for (int j = 0; j < (1 << R); j++) {
        if (j & (1 << LT)) continue;
        if ((uint32_t(j) & lcm) != lcv) continue;
        body1_sel<T, BODY, EMU>(mr, kr, a[j], a[j | (1 << LT)]);
    }
}

template <class T, int R, int BODY, bool EMU>
__device__ __forceinline__ void reg_gate_lt(cplx_t<T> (&a)[1 << R], int lt, const T *m, const KConst *k, uint32_t lcm,
                                            uint32_t lcv) {
    switch (lt) {
    case 0: reg_gate<T, R, 0, BODY, EMU>(a, m, k, lcm, lcv); break;
    case 1: reg_gate<T, R, 1, BODY, EMU>(a, m, k, lcm, lcv); break;
    case 2: reg_gate<T, R, 2 % R, BODY, EMU>(a, m, k, lcm, lcv); break;
    default: reg_gate<T, R, (R - 1), BODY, EMU>(a, m, k, lcm, lcv); break;
    }
}

template <class T, int R, bool EMU>
__device__ __forceinline__ void reg_gate_any(cplx_t<T> (&a)[1 << R], int body, int lt, const T *m, const KConst *k,
                                             uint32_t lcm, uint32_t lcv) {
    switch (body) {
    case B_DIAG: reg_gate_lt<T, R, B_DIAG, EMU>(a, lt, m, k, lcm, lcv); break;
    case B_PERM: reg_gate_lt<T, R, B_PERM, EMU>(a, lt, m, k, lcm, lcv); break;
    case B_ANTIDIAG: reg_gate_lt<T, R, B_ANTIDIAG, EMU>(a, lt, m, k, lcm, lcv); break;
    case B_REAL: reg_gate_lt<T, R, B_REAL, EMU>(a, lt, m, k, lcm, lcv); break;
    case B_RXLIKE: reg_gate_lt<T, R, B_RXLIKE, EMU>(a, lt, m, k, lcm, lcv); break;
    default: reg_gate_lt<T, R, B_DENSE, false>(a, lt, m, k, lcm, lcv); break;
    }
}

// Host: structured body of a 2x2 matrix (re/im interleaved, row-major) and
// the integer-pipe multipliers its complex128 body uses (lgpu_gates.cu).
int body_of_2x2_host(const double *m, KConst *kc);

}  // namespace lgpu
