// FP64 relief for complex128 kernels on GB300.
//
// GB300 issues about 2 FP64 FMAs per clock per SM (1.2 TFLOP/s), so a
// complex128 gate that needs 8 FP64 operations per amplitude pair is bound by
// the FP64 pipe well below HBM bandwidth.  emul() computes k * x for a double
// x and a host-prepared double constant k on the INTEGER pipe: the 53-bit
// mantissas are multiplied with 32x32->64-bit integer multiplies, the top 53
// bits of the 106-bit product are kept and rounded half-up on the first
// discarded bit, and the exponent is rebuilt.  The result equals the
// correctly rounded IEEE product except on exact ties (then it is one ulp
// away); zero and subnormal inputs or underflowing products return a signed
// zero (|result| < 2^-1022).
//
// Each output component of a structured gate body then costs one DFMA plus
// one emul() instead of two FP64 operations, halving FP64 issue pressure.
#pragma once

#include <stdint.h>

#include <cstring>

#if defined(__CUDACC__)
#define LGPU_HD __host__ __device__ __forceinline__
#else
#define LGPU_HD inline
#endif

namespace lgpu {

// Host/device portable bit casts and high product (the host versions let the
// arithmetic be unit-tested with a plain C++ compiler).
LGPU_HD uint64_t emu_bits(double x) {
#if defined(__CUDA_ARCH__)
    return static_cast<uint64_t>(__double_as_longlong(x));
#else
    uint64_t b;
    std::memcpy(&b, &x, sizeof(b));
    return b;
#endif
}
LGPU_HD double emu_double(uint64_t b) {
#if defined(__CUDA_ARCH__)
    return __longlong_as_double(static_cast<long long>(b));
#else
    double x;
    std::memcpy(&x, &b, sizeof(x));
    return x;
#endif
}
LGPU_HD uint32_t emu_umulhi(uint32_t a, uint32_t b) {
#if defined(__CUDA_ARCH__)
    return __umulhi(a, b);
#else
    return uint32_t((uint64_t(a) * b) >> 32);
#endif
}

struct KConst {
    uint32_t mh;    // mantissa bits 52..32 with the implicit one (21 bits); 0 when k == 0
    uint32_t ml;    // mantissa bits 31..0
    int32_t eadj;   // biased exponent of k minus 1023
    uint32_t sign;  // 0x80000000 when k < 0
};

LGPU_HD KConst make_kconst(double k) {
    KConst c{};
    const uint64_t b = emu_bits(k);
    const uint32_t hi = uint32_t(b >> 32), lo = uint32_t(b);
    const uint32_t e = (hi >> 20) & 0x7FF;
    c.sign = hi & 0x80000000u;
    if (e == 0) {  // zero (subnormal constants are treated as zero)
        c.mh = 0;
        c.ml = 0;
        c.eadj = -2000;
        return c;
    }
    c.mh = (hi & 0xFFFFFu) | 0x100000u;
    c.ml = lo;
    c.eadj = int32_t(e) - 1023;
    return c;
}

LGPU_HD double emul(double x, const KConst &k) {
    const uint64_t xb = emu_bits(x);
    const uint32_t xh = uint32_t(xb >> 32), xl = uint32_t(xb);
    const int32_t ex = int32_t((xh >> 20) & 0x7FFu);
    const uint32_t mh = (xh & 0xFFFFFu) | 0x100000u;
    // P = (mh*2^32 + xl) * (k.mh*2^32 + k.ml);  Q = P >> 32 = hh*2^32 + t  (exact)
    const uint64_t hh = uint64_t(mh) * k.mh;
    const uint64_t t = uint64_t(mh) * k.ml + uint64_t(xl) * k.mh + emu_umulhi(xl, k.ml);
    const uint64_t qhi = hh + (t >> 32);  // Q = qhi * 2^32 + qlo, Q in [2^72, 2^74)
    const uint32_t qlo = uint32_t(t);
    const bool top = (qhi >> 41) != 0;
    const int s = top ? 11 : 12;
    const uint64_t M = (qhi << s) | (uint64_t(qlo) >> (32 - s));  // 53-bit mantissa with implicit one
    const uint64_t rnd = (qlo >> (31 - s)) & 1u;
    const int32_t E = ex + k.eadj + (top ? 1 : 0);  // biased exponent of the result
    const uint64_t sign = uint64_t((xh ^ k.sign) & 0x80000000u) << 32;
    const uint64_t mag = (uint64_t(uint32_t(E - 1)) << 52) + M + rnd;
    const bool ok = (ex != 0) && (E > 0) && (k.mh != 0);
    return emu_double(sign | (ok ? mag : 0ull));
}

}  // namespace lgpu
