// Gate and generator matrices (same factory names as the reference
// src/simulator/cuGates_host.hpp:26-1326).  All matrices here are PennyLane
// row-major with the FIRST wire as the most significant matrix bit; the
// reference stores its named 2- and 4-qubit matrices with the first wire as
// the least significant bit and applies them without reversing the targets,
// which is the same operator.
#pragma once

#include <cmath>
#include <complex>
#include <vector>

#include "cuda_helpers.hpp"

namespace Pennylane::CUDA::cuGates {

template <class CFP_t> using Real = decltype(CFP_t{}.x);

template <class CFP_t> static auto c_(double re, double im = 0.0) -> CFP_t {
    return CFP_t{static_cast<Real<CFP_t>>(re), static_cast<Real<CFP_t>>(im)};
}
template <class CFP_t> static auto polar_(double theta) -> CFP_t { return c_<CFP_t>(std::cos(theta), std::sin(theta)); }

template <class CFP_t> static auto diag_(const std::vector<CFP_t> &d) -> std::vector<CFP_t> {
    const size_t D = d.size();
    std::vector<CFP_t> m(D * D, c_<CFP_t>(0));
    for (size_t i = 0; i < D; i++) m[i * D + i] = d[i];
    return m;
}

template <class CFP_t> static auto getIdentity() -> std::vector<CFP_t> { return {c_<CFP_t>(1), c_<CFP_t>(0), c_<CFP_t>(0), c_<CFP_t>(1)}; }
template <class CFP_t> static auto getPauliX() -> std::vector<CFP_t> { return {c_<CFP_t>(0), c_<CFP_t>(1), c_<CFP_t>(1), c_<CFP_t>(0)}; }
template <class CFP_t> static auto getPauliY() -> std::vector<CFP_t> { return {c_<CFP_t>(0), c_<CFP_t>(0, -1), c_<CFP_t>(0, 1), c_<CFP_t>(0)}; }
template <class CFP_t> static auto getPauliZ() -> std::vector<CFP_t> { return {c_<CFP_t>(1), c_<CFP_t>(0), c_<CFP_t>(0), c_<CFP_t>(-1)}; }
template <class CFP_t> static auto getHadamard() -> std::vector<CFP_t> {
    const double r = 1.0 / std::sqrt(2.0);
    return {c_<CFP_t>(r), c_<CFP_t>(r), c_<CFP_t>(r), c_<CFP_t>(-r)};
}
template <class CFP_t> static auto getS() -> std::vector<CFP_t> { return {c_<CFP_t>(1), c_<CFP_t>(0), c_<CFP_t>(0), c_<CFP_t>(0, 1)}; }
template <class CFP_t> static auto getT() -> std::vector<CFP_t> {
    return {c_<CFP_t>(1), c_<CFP_t>(0), c_<CFP_t>(0), polar_<CFP_t>(M_PI / 4)};
}

template <class CFP_t> static auto controlled_(const std::vector<CFP_t> &u, size_t nctrl) -> std::vector<CFP_t> {
    size_t du = 1;
    while (du * du < u.size()) du++;
    const size_t D = du << nctrl;
    std::vector<CFP_t> m(D * D, c_<CFP_t>(0));
    for (size_t i = 0; i < D - du; i++) m[i * D + i] = c_<CFP_t>(1);
    for (size_t r = 0; r < du; r++)
        for (size_t c = 0; c < du; c++) m[(D - du + r) * D + (D - du + c)] = u[r * du + c];
    return m;
}

template <class CFP_t> static auto getCNOT() -> std::vector<CFP_t> { return controlled_(getPauliX<CFP_t>(), 1); }
template <class CFP_t> static auto getSWAP() -> std::vector<CFP_t> {
    std::vector<CFP_t> m(16, c_<CFP_t>(0));
    m[0] = m[6] = m[9] = m[15] = c_<CFP_t>(1);
    return m;
}
template <class CFP_t> static auto getCY() -> std::vector<CFP_t> { return controlled_(getPauliY<CFP_t>(), 1); }
template <class CFP_t> static auto getCZ() -> std::vector<CFP_t> { return controlled_(getPauliZ<CFP_t>(), 1); }
template <class CFP_t> static auto getCSWAP() -> std::vector<CFP_t> { return controlled_(getSWAP<CFP_t>(), 1); }
template <class CFP_t> static auto getToffoli() -> std::vector<CFP_t> { return controlled_(getPauliX<CFP_t>(), 2); }

template <class CFP_t, class U = double> static auto getPhaseShift(U angle) -> std::vector<CFP_t> {
    return {c_<CFP_t>(1), c_<CFP_t>(0), c_<CFP_t>(0), polar_<CFP_t>(angle)};
}
template <class CFP_t, class U = double> static auto getPhaseShift(const std::vector<U> &p) -> std::vector<CFP_t> {
    return getPhaseShift<CFP_t>(p[0]);
}
template <class CFP_t, class U = double> static auto getRX(U angle) -> std::vector<CFP_t> {
    const double c = std::cos(angle / 2), s = std::sin(angle / 2);
    return {c_<CFP_t>(c), c_<CFP_t>(0, -s), c_<CFP_t>(0, -s), c_<CFP_t>(c)};
}
template <class CFP_t, class U = double> static auto getRX(const std::vector<U> &p) -> std::vector<CFP_t> { return getRX<CFP_t>(p[0]); }
template <class CFP_t, class U = double> static auto getRY(U angle) -> std::vector<CFP_t> {
    const double c = std::cos(angle / 2), s = std::sin(angle / 2);
    return {c_<CFP_t>(c), c_<CFP_t>(-s), c_<CFP_t>(s), c_<CFP_t>(c)};
}
template <class CFP_t, class U = double> static auto getRY(const std::vector<U> &p) -> std::vector<CFP_t> { return getRY<CFP_t>(p[0]); }
template <class CFP_t, class U = double> static auto getRZ(U angle) -> std::vector<CFP_t> {
    return {polar_<CFP_t>(-angle / 2.0), c_<CFP_t>(0), c_<CFP_t>(0), polar_<CFP_t>(angle / 2.0)};
}
template <class CFP_t, class U = double> static auto getRZ(const std::vector<U> &p) -> std::vector<CFP_t> { return getRZ<CFP_t>(p[0]); }
// Rot(phi, theta, omega) = RZ(omega) RY(theta) RZ(phi)
template <class CFP_t, class U = double> static auto getRot(U phi, U theta, U omega) -> std::vector<CFP_t> {
    const double c = std::cos(theta / 2), s = std::sin(theta / 2);
    const double p = double(phi) + omega, m = double(phi) - omega;
    return {c_<CFP_t>(c * std::cos(p / 2), -c * std::sin(p / 2)), c_<CFP_t>(-s * std::cos(m / 2), -s * std::sin(m / 2)),
            c_<CFP_t>(s * std::cos(m / 2), -s * std::sin(m / 2)), c_<CFP_t>(c * std::cos(p / 2), c * std::sin(p / 2))};
}
template <class CFP_t, class U = double> static auto getRot(const std::vector<U> &p) -> std::vector<CFP_t> {
    return getRot<CFP_t>(p[0], p[1], p[2]);
}
template <class CFP_t, class U = double> static auto getCRX(U a) -> std::vector<CFP_t> { return controlled_(getRX<CFP_t>(a), 1); }
template <class CFP_t, class U = double> static auto getCRY(U a) -> std::vector<CFP_t> { return controlled_(getRY<CFP_t>(a), 1); }
template <class CFP_t, class U = double> static auto getCRZ(U a) -> std::vector<CFP_t> { return controlled_(getRZ<CFP_t>(a), 1); }
template <class CFP_t, class U = double> static auto getCRot(U phi, U theta, U omega) -> std::vector<CFP_t> {
    return controlled_(getRot<CFP_t>(phi, theta, omega), 1);
}
template <class CFP_t, class U = double> static auto getControlledPhaseShift(U a) -> std::vector<CFP_t> {
    return controlled_(getPhaseShift<CFP_t>(a), 1);
}

template <class CFP_t> static auto singleExcitation_(double angle, CFP_t outer) -> std::vector<CFP_t> {
    const double c = std::cos(angle / 2), s = std::sin(angle / 2);
    std::vector<CFP_t> m(16, c_<CFP_t>(0));
    m[0] = outer;
    m[5] = c_<CFP_t>(c);
    m[6] = c_<CFP_t>(-s);
    m[9] = c_<CFP_t>(s);
    m[10] = c_<CFP_t>(c);
    m[15] = outer;
    return m;
}
template <class CFP_t, class U = double> static auto getSingleExcitation(U a) -> std::vector<CFP_t> {
    return singleExcitation_<CFP_t>(a, c_<CFP_t>(1));
}
template <class CFP_t, class U = double> static auto getSingleExcitationMinus(U a) -> std::vector<CFP_t> {
    return singleExcitation_<CFP_t>(a, polar_<CFP_t>(-a / 2.0));
}
template <class CFP_t, class U = double> static auto getSingleExcitationPlus(U a) -> std::vector<CFP_t> {
    return singleExcitation_<CFP_t>(a, polar_<CFP_t>(a / 2.0));
}
template <class CFP_t> static auto genSingleExcitation_(double outer) -> std::vector<CFP_t> {
    std::vector<CFP_t> m(16, c_<CFP_t>(0));
    m[0] = c_<CFP_t>(outer);
    m[15] = c_<CFP_t>(outer);
    m[1 * 4 + 2] = c_<CFP_t>(0, -1);
    m[2 * 4 + 1] = c_<CFP_t>(0, 1);
    return m;
}
template <class CFP_t, class U = double> static auto getGeneratorSingleExcitation() -> std::vector<CFP_t> { return genSingleExcitation_<CFP_t>(0.0); }
template <class CFP_t, class U = double> static auto getGeneratorSingleExcitationMinus() -> std::vector<CFP_t> { return genSingleExcitation_<CFP_t>(1.0); }
template <class CFP_t, class U = double> static auto getGeneratorSingleExcitationPlus() -> std::vector<CFP_t> { return genSingleExcitation_<CFP_t>(-1.0); }

template <class CFP_t> static auto doubleExcitation_(double angle, CFP_t outer) -> std::vector<CFP_t> {
    const double c = std::cos(angle / 2), s = std::sin(angle / 2);
    std::vector<CFP_t> m(256, c_<CFP_t>(0));
    for (int i = 0; i < 16; i++) m[size_t(i * 16 + i)] = outer;
    m[3 * 16 + 3] = c_<CFP_t>(c);
    m[3 * 16 + 12] = c_<CFP_t>(-s);
    m[12 * 16 + 3] = c_<CFP_t>(s);
    m[12 * 16 + 12] = c_<CFP_t>(c);
    return m;
}
template <class CFP_t, class U = double> static auto getDoubleExcitation(U a) -> std::vector<CFP_t> {
    return doubleExcitation_<CFP_t>(a, c_<CFP_t>(1));
}
template <class CFP_t, class U = double> static auto getDoubleExcitationMinus(U a) -> std::vector<CFP_t> {
    return doubleExcitation_<CFP_t>(a, polar_<CFP_t>(-a / 2.0));
}
template <class CFP_t, class U = double> static auto getDoubleExcitationPlus(U a) -> std::vector<CFP_t> {
    return doubleExcitation_<CFP_t>(a, polar_<CFP_t>(a / 2.0));
}
template <class CFP_t> static auto genDoubleExcitation_(double outer) -> std::vector<CFP_t> {
    std::vector<CFP_t> m(256, c_<CFP_t>(0));
    for (int i = 0; i < 16; i++)
        if (i != 3 && i != 12) m[size_t(i * 16 + i)] = c_<CFP_t>(outer);
    m[3 * 16 + 12] = c_<CFP_t>(0, -1);
    m[12 * 16 + 3] = c_<CFP_t>(0, 1);
    return m;
}
template <class CFP_t, class U = double> static auto getGeneratorDoubleExcitation() -> std::vector<CFP_t> { return genDoubleExcitation_<CFP_t>(0.0); }
template <class CFP_t, class U = double> static auto getGeneratorDoubleExcitationMinus() -> std::vector<CFP_t> { return genDoubleExcitation_<CFP_t>(1.0); }
template <class CFP_t, class U = double> static auto getGeneratorDoubleExcitationPlus() -> std::vector<CFP_t> { return genDoubleExcitation_<CFP_t>(-1.0); }

template <class CFP_t, class U = double> static auto getIsingXX(U angle) -> std::vector<CFP_t> {
    const double c = std::cos(angle / 2), s = std::sin(angle / 2);
    std::vector<CFP_t> m(16, c_<CFP_t>(0));
    m[0] = m[5] = m[10] = m[15] = c_<CFP_t>(c);
    m[3] = m[6] = m[9] = m[12] = c_<CFP_t>(0, -s);
    return m;
}
template <class CFP_t, class U = double> static auto getIsingYY(U angle) -> std::vector<CFP_t> {
    const double c = std::cos(angle / 2), s = std::sin(angle / 2);
    std::vector<CFP_t> m(16, c_<CFP_t>(0));
    m[0] = m[5] = m[10] = m[15] = c_<CFP_t>(c);
    m[3] = m[12] = c_<CFP_t>(0, s);
    m[6] = m[9] = c_<CFP_t>(0, -s);
    return m;
}
template <class CFP_t, class U = double> static auto getIsingZZ(U angle) -> std::vector<CFP_t> {
    return diag_<CFP_t>({polar_<CFP_t>(-angle / 2.0), polar_<CFP_t>(angle / 2.0), polar_<CFP_t>(angle / 2.0),
                         polar_<CFP_t>(-angle / 2.0)});
}
template <class CFP_t, class U = double> static auto getGeneratorIsingXX() -> std::vector<CFP_t> {
    std::vector<CFP_t> m(16, c_<CFP_t>(0));
    m[3] = m[6] = m[9] = m[12] = c_<CFP_t>(1);
    return m;
}
template <class CFP_t, class U = double> static auto getGeneratorIsingYY() -> std::vector<CFP_t> {
    std::vector<CFP_t> m(16, c_<CFP_t>(0));
    m[6] = m[9] = c_<CFP_t>(1);
    m[3] = m[12] = c_<CFP_t>(-1);
    return m;
}
template <class CFP_t, class U = double> static auto getGeneratorIsingZZ() -> std::vector<CFP_t> {
    return diag_<CFP_t>({c_<CFP_t>(1), c_<CFP_t>(-1), c_<CFP_t>(-1), c_<CFP_t>(1)});
}

// Projectors used by the PhaseShift generators (GateGenerators.hpp:23-56).
template <class CFP_t> static auto getP11_CU() -> std::vector<CFP_t> { return {c_<CFP_t>(0), c_<CFP_t>(0), c_<CFP_t>(0), c_<CFP_t>(1)}; }
template <class CFP_t> static auto getP1111_CU() -> std::vector<CFP_t> {
    return diag_<CFP_t>({c_<CFP_t>(0), c_<CFP_t>(0), c_<CFP_t>(0), c_<CFP_t>(1)});
}

} // namespace Pennylane::CUDA::cuGates
