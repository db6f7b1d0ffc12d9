// Gate application for the host tests of the engine's lowering: a lowered
// GateDesc applied to a full state vector by dense matrix-vector products.
#pragma once

#include <complex>
#include <cstdint>
#include <vector>

#include "GateLowering.hpp"

namespace hosttest {

using namespace Pennylane::Engine;
using cdv = std::vector<std::complex<double>>;

// Dense 2^t x 2^t matrix on target bits tg (tg[0] = most significant matrix
// bit) under controls ct with values cv.
inline void apply_dense(cdv &sv, const std::vector<int> &tg, const std::vector<int> &ct, const std::vector<int> &cv,
                        const cdv &m) {
    const size_t t = tg.size(), D = size_t(1) << t;
    uint64_t tmask = 0;
    for (int b : tg) tmask |= uint64_t(1) << b;
    std::vector<size_t> off(D);
    for (size_t r = 0; r < D; r++) {
        size_t o = 0;
        for (size_t k = 0; k < t; k++)
            if ((r >> (t - 1 - k)) & 1) o |= size_t(1) << tg[k];
        off[r] = o;
    }
    cdv a(D), y(D);
    for (size_t i = 0; i < sv.size(); i++) {
        if (i & tmask) continue;
        bool on = true;
        for (size_t k = 0; k < ct.size(); k++)
            if (int((i >> ct[k]) & 1) != cv[k]) on = false;
        if (!on) continue;
        for (size_t c = 0; c < D; c++) a[c] = sv[i | off[c]];
        for (size_t r = 0; r < D; r++) {
            std::complex<double> s = 0;
            for (size_t c = 0; c < D; c++) s += m[r * D + c] * a[c];
            y[r] = s;
        }
        for (size_t r = 0; r < D; r++) sv[i | off[r]] = y[r];
    }
}

inline bool apply_desc(cdv &sv, const GateDesc &d) {
    if (d.kind == GateDesc::IDENTITY) return true;
    if (d.kind == GateDesc::MATRIX) {
        std::vector<int> cv = d.cvals;
        if (cv.empty()) cv.assign(d.ctrls.size(), 1);
        apply_dense(sv, d.tgts, d.ctrls, cv, d.matrix);
        return true;
    }
    std::vector<int> bits;
    cdv m;
    if (!dense_on_bits(d, bits, m, 12)) return false;
    apply_dense(sv, bits, {}, {}, m);
    return true;
}


}  // namespace hosttest
