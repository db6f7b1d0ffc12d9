// ORACLE — test infrastructure only.
//
// A CPU restatement (C++17, OpenMP) of the semantics of the reference
// statevector engine (PennyLane-Lightning-GPU 0.33.0-dev).  It is the checker
// for the CUDA path and the timed CPU baseline; nothing in the product links,
// imports or calls it.  Every function names the reference file:line whose
// behaviour it restates.  The reference's arithmetic lives in the closed
// cuStateVec / cuBLAS / cuSPARSE libraries, so the oracle restates the
// published mathematics of those calls (matrix application, Pauli rotation,
// expectation, marginal probabilities, inverse-CDF sampling, zdotc/zaxpy,
// CSR SpMV) with the reference's conventions:
//   * wire w <-> state-index bit (n-1-w)     StateVectorCudaManaged.hpp:1349-1356
//   * matrices are PennyLane row-major with wires[0] as the most significant
//     matrix bit (named 2-qubit gates of cuGates_host.hpp are stored LSB-first
//     and applied with targets NOT reversed, which is the same operator;
//     user matrices are applied with targets reversed,
//     StateVectorCudaManaged.hpp:231-245)
//   * controls are the first ctrl_map[name] wires   StateVectorCudaBase.hpp:288-312
//   * Pauli rotations apply exp(-i*param/2*P) (adjoint: +)   StateVectorCudaManaged.hpp:1372
#pragma once

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <map>
#include <random>
#include <stdexcept>
#include <string>
#include <vector>

namespace oracle {

using cd = std::complex<double>;
using Mat = std::vector<cd>;

struct OracleError : std::runtime_error {
    using std::runtime_error::runtime_error;
};

inline int bit_of_wire(int n, int w) { return n - 1 - w; }

// ---------------------------------------------------------------------------
// Gate matrices, PennyLane convention (cuGates_host.hpp:26-1326 restated in
// MSB-first order; cuGateCache.hpp:60-161 for the constant gates).
// ---------------------------------------------------------------------------
inline Mat mat_identity(int dim) {
    Mat m(dim * dim, 0.0);
    for (int i = 0; i < dim; i++) m[i * dim + i] = 1.0;
    return m;
}
inline Mat m_paulix() { return {0, 1, 1, 0}; }
inline Mat m_pauliy() { return {0, cd(0, -1), cd(0, 1), 0}; }
inline Mat m_pauliz() { return {1, 0, 0, -1}; }
inline Mat m_hadamard() {
    const double r = 1.0 / std::sqrt(2.0);
    return {r, r, r, -r};
}
inline Mat m_s() { return {1, 0, 0, cd(0, 1)}; }
inline Mat m_t() { return {1, 0, 0, std::polar(1.0, M_PI / 4)}; }
inline Mat m_swap() { return {1, 0, 0, 0, 0, 0, 1, 0, 0, 1, 0, 0, 0, 0, 0, 1}; }
inline Mat m_phaseshift(double p) { return {1, 0, 0, std::polar(1.0, p)}; }
inline Mat m_rx(double t) {
    const double c = std::cos(t / 2), s = std::sin(t / 2);
    return {c, cd(0, -s), cd(0, -s), c};
}
inline Mat m_ry(double t) {
    const double c = std::cos(t / 2), s = std::sin(t / 2);
    return {c, -s, s, c};
}
inline Mat m_rz(double t) {
    return {std::polar(1.0, -t / 2), 0, 0, std::polar(1.0, t / 2)};
}
// Rot(phi, theta, omega) = RZ(omega) RY(theta) RZ(phi)   cuGates_host.hpp:390-422
inline Mat m_rot(double phi, double theta, double omega) {
    const double c = std::cos(theta / 2), s = std::sin(theta / 2);
    const double p = phi + omega, m = phi - omega;
    return {c * std::polar(1.0, -p / 2), -s * std::polar(1.0, m / 2),
            s * std::polar(1.0, -m / 2), c * std::polar(1.0, p / 2)};
}
// cuGates_host.hpp:639-670 (stored LSB-first there)
inline Mat m_single_excitation(double t, cd outer) {
    const double c = std::cos(t / 2), s = std::sin(t / 2);
    return {outer, 0, 0, 0, 0, c, -s, 0, 0, s, c, 0, 0, 0, 0, outer};
}
// cuGates_host.hpp:870-905 (stored LSB-first there)
inline Mat m_double_excitation(double t, cd outer) {
    const double c = std::cos(t / 2), s = std::sin(t / 2);
    Mat m(256, 0.0);
    for (int i = 0; i < 16; i++) m[i * 16 + i] = outer;
    m[3 * 16 + 3] = c;
    m[3 * 16 + 12] = -s;
    m[12 * 16 + 3] = s;
    m[12 * 16 + 12] = c;
    return m;
}
// Generators (cuGates_host.hpp:686-712, 764-791, 843-868, 921-938, 994-1026,
// 1082-1112, 1160-1185, 1213-1240, 1270-1295; GateGenerators.hpp:90-160).
inline Mat m_gen_single_excitation(cd outer) {
    Mat m(16, 0.0);
    m[0] = outer;
    m[15] = outer;
    m[1 * 4 + 2] = cd(0, -1);
    m[2 * 4 + 1] = cd(0, 1);
    return m;
}
inline Mat m_gen_double_excitation(cd outer) {
    Mat m(256, 0.0);
    for (int i = 0; i < 16; i++)
        if (i != 3 && i != 12) m[i * 16 + i] = outer;
    m[3 * 16 + 12] = cd(0, -1);
    m[12 * 16 + 3] = cd(0, 1);
    return m;
}
inline Mat kron(const Mat &a, int da, const Mat &b, int db) {
    Mat m(da * db * da * db);
    for (int i = 0; i < da; i++)
        for (int j = 0; j < da; j++)
            for (int k = 0; k < db; k++)
                for (int l = 0; l < db; l++)
                    m[(i * db + k) * (da * db) + (j * db + l)] = a[i * da + j] * b[k * db + l];
    return m;
}
inline Mat dagger(const Mat &m, int dim) {
    Mat r(dim * dim);
    for (int i = 0; i < dim; i++)
        for (int j = 0; j < dim; j++) r[i * dim + j] = std::conj(m[j * dim + i]);
    return r;
}

// ---------------------------------------------------------------------------
// Index helpers
// ---------------------------------------------------------------------------
inline uint64_t insert_zero_bits(uint64_t g, const std::vector<int> &sorted_bits) {
    for (int b : sorted_bits) {
        const uint64_t lo = g & ((uint64_t(1) << b) - 1);
        g = ((g >> b) << (b + 1)) | lo;
    }
    return g;
}

template <class P> struct State {
    int n = 0;
    std::vector<std::complex<P>> a;
    explicit State(int nq) : n(nq), a(size_t(1) << nq, 0.0) { a[0] = 1.0; }
};

// ---------------------------------------------------------------------------
// Dense controlled matrix application (custatevecApplyMatrix restated;
// StateVectorCudaManaged.hpp:1400-1472, 1484-1556).  Matrix index bit (t-1-k)
// corresponds to tgt_wires[k]; every control wire must be |1>.
// ---------------------------------------------------------------------------
template <class P>
void apply_matrix(std::vector<std::complex<P>> &sv, int n, const Mat &m,
                  const std::vector<int> &ctrl_wires, const std::vector<int> &tgt_wires) {
    const int t = int(tgt_wires.size());
    const int dim = 1 << t;
    if (int(m.size()) != dim * dim) throw OracleError("matrix size does not match target count");
    std::vector<int> bits;
    uint64_t cmask = 0;
    for (int w : ctrl_wires) {
        bits.push_back(bit_of_wire(n, w));
        cmask |= uint64_t(1) << bit_of_wire(n, w);
    }
    std::vector<uint64_t> off(dim, 0);
    for (int k = 0; k < t; k++) bits.push_back(bit_of_wire(n, tgt_wires[k]));
    for (int r = 0; r < dim; r++)
        for (int k = 0; k < t; k++)
            if ((r >> (t - 1 - k)) & 1) off[r] |= uint64_t(1) << bit_of_wire(n, tgt_wires[k]);
    std::sort(bits.begin(), bits.end());
    if (std::adjacent_find(bits.begin(), bits.end()) != bits.end())
        throw OracleError("repeated wire");
    const int64_t ngroups = int64_t(1) << (n - int(bits.size()));
    if (t == 1) {
        // the same arithmetic as the general loop below, without its per-group buffers
        const uint64_t o1 = off[1];
        const cd m00 = m[0], m01 = m[1], m10 = m[2], m11 = m[3];
#pragma omp parallel for schedule(static)
        for (int64_t g = 0; g < ngroups; g++) {
            const uint64_t base = insert_zero_bits(uint64_t(g), bits) | cmask;
            const std::complex<double> x(sv[base]), y(sv[base | o1]);
            std::complex<double> r0 = 0, r1 = 0;
            r0 += m00 * x;
            r0 += m01 * y;
            r1 += m10 * x;
            r1 += m11 * y;
            sv[base] = std::complex<P>(r0);
            sv[base | o1] = std::complex<P>(r1);
        }
        return;
    }
#pragma omp parallel
    {
        std::vector<std::complex<P>> in(dim), out(dim);
#pragma omp for schedule(static)
        for (int64_t g = 0; g < ngroups; g++) {
            const uint64_t base = insert_zero_bits(uint64_t(g), bits) | cmask;
            for (int r = 0; r < dim; r++) in[r] = sv[base | off[r]];
            for (int r = 0; r < dim; r++) {
                std::complex<double> acc = 0;
                for (int c = 0; c < dim; c++)
                    acc += m[r * dim + c] * std::complex<double>(in[c]);
                out[r] = std::complex<P>(acc);
            }
            for (int r = 0; r < dim; r++) sv[base | off[r]] = out[r];
        }
    }
}

// ---------------------------------------------------------------------------
// Pauli rotation exp(i*angle*P), P a Pauli word on tgt_wires, controls |1>
// (custatevecApplyPauliRotation; StateVectorCudaManaged.hpp:1339-1386).
// P|j> = i^{nY} (-1)^{popcount(j & (Y|Z mask))} |j ^ (X|Y mask)>.
// ---------------------------------------------------------------------------
template <class P>
void apply_pauli_rotation(std::vector<std::complex<P>> &sv, int n, double angle,
                          const std::string &paulis, const std::vector<int> &ctrl_wires,
                          const std::vector<int> &tgt_wires) {
    uint64_t flip = 0, sgn = 0, cmask = 0;
    int ny = 0;
    for (size_t k = 0; k < tgt_wires.size(); k++) {
        const uint64_t b = uint64_t(1) << bit_of_wire(n, tgt_wires[k]);
        switch (paulis[k]) {
        case 'X': flip |= b; break;
        case 'Y': flip |= b; sgn |= b; ny++; break;
        case 'Z': sgn |= b; break;
        case 'I': break;
        default: throw OracleError("bad Pauli letter");
        }
    }
    for (int w : ctrl_wires) cmask |= uint64_t(1) << bit_of_wire(n, w);
    const cd iny[4] = {1.0, cd(0, 1), -1.0, cd(0, -1)};
    const cd ph = iny[ny & 3];
    const double c = std::cos(angle), s = std::sin(angle);
    const int64_t N = int64_t(1) << n;
    // (P a)_i = ph * sign(j) * a_j with j = i ^ flip; exp(i angle P) a = c a + i s P a.
    // Computed in place: amplitudes i and j = i ^ flip depend only on each other.
    auto out_of = [&](uint64_t i, const cd &ai, const cd &aj) {
        const uint64_t j = i ^ flip;
        const double sign = (__builtin_popcountll(j & sgn) & 1) ? -1.0 : 1.0;
        const cd pa = ph * sign * aj;
        return std::complex<P>(c * ai + cd(0, s) * pa);
    };
    if (flip == 0) {
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < N; i++) {
            if ((uint64_t(i) & cmask) != cmask) continue;
            const cd a = cd(sv[size_t(i)]);
            sv[size_t(i)] = out_of(uint64_t(i), a, a);
        }
        return;
    }
    const int hb = 63 - __builtin_clzll(flip);
    const uint64_t lo = (uint64_t(1) << hb) - 1;
#pragma omp parallel for schedule(static)
    for (int64_t g = 0; g < N / 2; g++) {
        const uint64_t i = ((uint64_t(g) & ~lo) << 1) | (uint64_t(g) & lo);  // bit hb of i is 0
        if ((i & cmask) != cmask) continue;
        const uint64_t j = i ^ flip;
        const cd ai = cd(sv[i]), aj = cd(sv[j]);
        sv[i] = out_of(i, ai, aj);
        sv[j] = out_of(j, aj, ai);
    }
}

// ---------------------------------------------------------------------------
// Operation dispatcher: StateVectorCudaManaged::applyOperation
// (StateVectorCudaManaged.hpp:198-247) with the per-gate methods it reaches
// (:320-560, :1179-1305) and the control map (StateVectorCudaBase.hpp:288-312).
// ---------------------------------------------------------------------------
inline const std::map<std::string, int> &ctrl_map() {
    static const std::map<std::string, int> m{
        {"Identity", 0}, {"PauliX", 0}, {"PauliY", 0}, {"PauliZ", 0}, {"Hadamard", 0},
        {"T", 0},        {"S", 0},      {"RX", 0},     {"RY", 0},     {"RZ", 0},
        {"Rot", 0},      {"PhaseShift", 0}, {"ControlledPhaseShift", 1}, {"CNOT", 1},
        {"SWAP", 0},     {"CY", 1},     {"CZ", 1},     {"CRX", 1},    {"CRY", 1},
        {"CRZ", 1},      {"CRot", 1},   {"CSWAP", 1},  {"Toffoli", 2}};
    return m;
}

// When true, Adjoint(Rot/CRot) follows the reference's literal behaviour
// (getRot(omega, theta, phi) daggered, StateVectorCudaManaged.hpp:215-224),
// which is not the inverse of Rot(phi, theta, omega) when phi != omega.  The
// default (false) applies the mathematical inverse.
inline bool &rot_adjoint_reference_quirk() {
    static bool q = false;
    return q;
}

template <class P>
void apply_operation(std::vector<std::complex<P>> &sv, int n, const std::string &name,
                     const std::vector<int> &wires, bool adj, const std::vector<double> &params,
                     const Mat &gate_matrix) {
    for (int w : wires)
        if (w < 0 || w >= n) throw OracleError("wire index out of range");
    const auto it = ctrl_map().find(name);
    const int nc = (it == ctrl_map().end()) ? 0 : it->second;
    if (int(wires.size()) < nc) throw OracleError("too few wires for " + name);
    const std::vector<int> ctrls(wires.begin(), wires.begin() + nc);
    const std::vector<int> tgts(wires.begin() + nc, wires.end());
    auto P0 = [&](int i) {
        if (int(params.size()) <= i) throw OracleError("missing parameter for " + name);
        return params[size_t(i)];
    };
    auto apply_m = [&](Mat m, const std::vector<int> &c, const std::vector<int> &t) {
        const int dim = 1 << t.size();
        if (adj) m = dagger(m, dim);
        apply_matrix(sv, n, m, c, t);
    };
    // Per-gate methods use ctrls = wires[:-1], tgts = {wires.back()}
    // (StateVectorCudaManaged.hpp:324-560).
    const std::vector<int> head(wires.begin(), wires.end() - (wires.empty() ? 0 : 1));
    const std::vector<int> last(wires.empty() ? wires.end() : wires.end() - 1, wires.end());

    if (name == "Identity" || name == "I") return;
    if (name == "RX" || name == "RY" || name == "RZ" || name == "CRX" || name == "CRY" ||
        name == "CRZ") {
        const char p = name.back();
        const double ang = adj ? P0(0) / 2 : -P0(0) / 2;
        apply_pauli_rotation(sv, n, ang, std::string(1, p), ctrls, tgts);
        return;
    }
    if (name == "Rot" || name == "CRot") {
        Mat m;
        if (adj && rot_adjoint_reference_quirk())
            m = m_rot(P0(2), P0(1), P0(0));
        else
            m = m_rot(P0(0), P0(1), P0(2));
        apply_m(m, ctrls, tgts);
        return;
    }
    if (name == "PhaseShift" || name == "ControlledPhaseShift") {
        apply_m(m_phaseshift(P0(0)), head, last);
        return;
    }
    if (name == "MultiRZ" || name == "IsingXX" || name == "IsingYY" || name == "IsingZZ") {
        const char p = (name == "MultiRZ") ? 'Z' : name.back();
        const double ang = adj ? P0(0) / 2 : -P0(0) / 2;
        apply_pauli_rotation(sv, n, ang, std::string(wires.size(), p), {}, wires);
        return;
    }
    if (name == "SingleExcitation" || name == "SingleExcitationMinus" ||
        name == "SingleExcitationPlus") {
        cd outer = 1.0;
        if (name == "SingleExcitationMinus") outer = std::polar(1.0, -P0(0) / 2);
        if (name == "SingleExcitationPlus") outer = std::polar(1.0, P0(0) / 2);
        apply_m(m_single_excitation(P0(0), outer), {}, wires);
        return;
    }
    if (name == "DoubleExcitation" || name == "DoubleExcitationMinus" ||
        name == "DoubleExcitationPlus") {
        cd outer = 1.0;
        if (name == "DoubleExcitationMinus") outer = std::polar(1.0, -P0(0) / 2);
        if (name == "DoubleExcitationPlus") outer = std::polar(1.0, P0(0) / 2);
        apply_m(m_double_excitation(P0(0), outer), {}, wires);
        return;
    }
    // constant gates from the gate cache (cuGateCache.hpp:60-161)
    if (name == "PauliX" || name == "CNOT" || name == "Toffoli") { apply_m(m_paulix(), ctrls, tgts); return; }
    if (name == "PauliY" || name == "CY") { apply_m(m_pauliy(), ctrls, tgts); return; }
    if (name == "PauliZ" || name == "CZ") { apply_m(m_pauliz(), ctrls, tgts); return; }
    if (name == "Hadamard") { apply_m(m_hadamard(), ctrls, tgts); return; }
    if (name == "S") { apply_m(m_s(), ctrls, tgts); return; }
    if (name == "T") { apply_m(m_t(), ctrls, tgts); return; }
    if (name == "SWAP" || name == "CSWAP") { apply_m(m_swap(), ctrls, tgts); return; }
    // generators (StateVectorCudaManaged.hpp:563-688; GateGenerators.hpp)
    if (name == "GeneratorIsingXX") { apply_m(kron(m_paulix(), 2, m_paulix(), 2), {}, wires); return; }
    if (name == "GeneratorIsingYY") { apply_m(kron(m_pauliy(), 2, m_pauliy(), 2), {}, wires); return; }
    if (name == "GeneratorIsingZZ") { apply_m(kron(m_pauliz(), 2, m_pauliz(), 2), {}, wires); return; }
    if (name == "GeneratorSingleExcitation") { apply_m(m_gen_single_excitation(0.0), {}, wires); return; }
    if (name == "GeneratorSingleExcitationMinus") { apply_m(m_gen_single_excitation(1.0), {}, wires); return; }
    if (name == "GeneratorSingleExcitationPlus") { apply_m(m_gen_single_excitation(-1.0), {}, wires); return; }
    if (name == "GeneratorDoubleExcitation") { apply_m(m_gen_double_excitation(0.0), {}, wires); return; }
    if (name == "GeneratorDoubleExcitationMinus") { apply_m(m_gen_double_excitation(1.0), {}, wires); return; }
    if (name == "GeneratorDoubleExcitationPlus") { apply_m(m_gen_double_excitation(-1.0), {}, wires); return; }
    if (name == "GeneratorMultiRZ") {
        for (int w : wires) apply_matrix(sv, n, m_pauliz(), {}, {w});
        return;
    }
    // gate_matrix fallback (StateVectorCudaManaged.hpp:231-245)
    if (gate_matrix.empty()) throw OracleError("Currently unsupported gate: " + name);
    apply_m(gate_matrix, ctrls, tgts);
}

// ---------------------------------------------------------------------------
// Measurements
// ---------------------------------------------------------------------------
// <psi|M|psi> for a dense matrix on wires (custatevecComputeExpectation;
// StateVectorCudaManaged.hpp:702-780, 1602-1713).
template <class P>
cd expval_matrix(const std::vector<std::complex<P>> &sv, int n, const Mat &m,
                 const std::vector<int> &wires) {
    std::vector<std::complex<P>> tmp(sv);
    apply_matrix(tmp, n, m, {}, wires);
    double re = 0, im = 0;
    const int64_t N = int64_t(1) << n;
#pragma omp parallel for reduction(+ : re, im) schedule(static)
    for (int64_t i = 0; i < N; i++) {
        const cd v = std::conj(cd(sv[i])) * cd(tmp[i]);
        re += v.real();
        im += v.imag();
    }
    return {re, im};
}

// sum_j Re(c_j <P_j>) (custatevecComputeExpectationsOnPauliBasis + host sum;
// StateVectorCudaManaged.hpp:1071-1148).  <P_j> is evaluated in double.
template <class P>
double expval_pauli_words(const std::vector<std::complex<P>> &sv, int n,
                          const std::vector<std::string> &words,
                          const std::vector<std::vector<int>> &word_wires,
                          const std::vector<cd> &coeffs) {
    const int64_t N = int64_t(1) << n;
    cd total = 0;
    const cd iny[4] = {1.0, cd(0, 1), -1.0, cd(0, -1)};
    for (size_t t = 0; t < words.size(); t++) {
        uint64_t flip = 0, sgn = 0;
        int ny = 0;
        for (size_t k = 0; k < word_wires[t].size(); k++) {
            const uint64_t b = uint64_t(1) << bit_of_wire(n, word_wires[t][k]);
            const char c = words[t][k];
            if (c == 'X') flip |= b;
            else if (c == 'Y') { flip |= b; sgn |= b; ny++; }
            else if (c == 'Z') sgn |= b;
            else if (c != 'I') throw OracleError("bad Pauli letter");
        }
        double re = 0, im = 0;
#pragma omp parallel for reduction(+ : re, im) schedule(static)
        for (int64_t i = 0; i < N; i++) {
            const uint64_t j = uint64_t(i) ^ flip;
            const double sign = (__builtin_popcountll(j & sgn) & 1) ? -1.0 : 1.0;
            const cd v = std::conj(cd(sv[i])) * sign * cd(sv[j]);
            re += v.real();
            im += v.imag();
        }
        const double ev = (iny[ny & 3] * cd(re, im)).real();
        total += ev * coeffs[t];
    }
    return total.real();
}

// Marginal probabilities; output bit k <-> wires[k] (custatevecAbs2SumArray;
// StateVectorCudaManaged.hpp:931-970).
template <class P>
std::vector<double> probability(const std::vector<std::complex<P>> &sv, int n,
                                const std::vector<int> &wires) {
    const int k = int(wires.size());
    std::vector<double> out(size_t(1) << k, 0.0);
    const int64_t N = int64_t(1) << n;
    for (int64_t i = 0; i < N; i++) {
        size_t idx = 0;
        for (int q = 0; q < k; q++) idx |= size_t((uint64_t(i) >> bit_of_wire(n, wires[q])) & 1) << q;
        out[idx] += std::norm(cd(sv[i]));
    }
    return out;
}

// Random numbers of the sampler: std::mt19937(seed) with
// std::uniform_real_distribution<DrawT>(0, 1) (StateVectorCudaManaged.hpp:1003-1007;
// the reference seeds from std::random_device, here the seed is explicit).
template <class DrawT> std::vector<double> sampler_draws(uint64_t seed, size_t shots) {
    std::mt19937 gen(static_cast<std::mt19937::result_type>(seed));
    std::uniform_real_distribution<DrawT> dis(0.0, 1.0);
    std::vector<double> r(shots);
    for (size_t i = 0; i < shots; i++) r[i] = double(dis(gen));
    return r;
}

// Inverse-CDF sampling with ascending output (custatevecSampler* with
// CUSTATEVEC_SAMPLER_OUTPUT_ASCENDING_ORDER; StateVectorCudaManaged.hpp:982-1061).
// Index for draw r: the smallest i with cdf_i > r * total; a draw at or past the
// end selects the last index of non-zero probability.
template <class P>
std::vector<uint64_t> sample_indices(const std::vector<std::complex<P>> &sv, int n,
                                     const std::vector<double> &draws) {
    const size_t N = size_t(1) << n;
    std::vector<double> cdf(N);
    double acc = 0;
    size_t last_nz = 0;
    for (size_t i = 0; i < N; i++) {
        const double p = std::norm(cd(sv[i]));
        acc += p;
        cdf[i] = acc;
        if (p > 0) last_nz = i;
    }
    std::vector<uint64_t> out(draws.size());
    for (size_t s = 0; s < draws.size(); s++) {
        const double target = draws[s] * acc;
        size_t i = size_t(std::upper_bound(cdf.begin(), cdf.end(), target) - cdf.begin());
        if (i >= N) i = last_nz;
        out[s] = i;
    }
    std::sort(out.begin(), out.end());
    return out;
}

// Host decode samples[s*n + (n-1-j)] = (idx >> j) & 1 (StateVectorCudaManaged.hpp:1038-1055).
inline std::vector<uint64_t> decode_samples(const std::vector<uint64_t> &idx, int n) {
    std::vector<uint64_t> out(idx.size() * size_t(n));
    for (size_t s = 0; s < idx.size(); s++)
        for (int j = 0; j < n; j++) out[s * n + (n - 1 - j)] = (idx[s] >> j) & 1;
    return out;
}

// ---------------------------------------------------------------------------
// Observables (ObservablesGPU.hpp:88-391): a term list with factors.
// ---------------------------------------------------------------------------
struct Factor {
    std::string name;          // PauliX/PauliY/PauliZ/Hadamard/Identity/... or "Hermitian"
    std::vector<int> wires;
    Mat matrix;                // used when non-empty
};
struct Term {
    double coeff = 1.0;
    std::vector<Factor> factors;
};
struct Observable {
    std::vector<Term> terms;   // one term with coeff 1: Named / Hermitian / TensorProd
    bool is_hamiltonian = false;
};

// dst = src with the host's threads (large states; same values as a copy).
template <class P>
void par_copy(std::vector<std::complex<P>> &dst, const std::vector<std::complex<P>> &src) {
    dst.resize(src.size());
    const int64_t N = int64_t(src.size());
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < N; i++) dst[size_t(i)] = src[size_t(i)];
}

// applyInPlace: Named -> applyOperation(name); Hermitian -> matrix;
// TensorProd -> sequential; Hamiltonian -> sum_t c_t O_t|psi>
// (ObservablesGPU.hpp:119-127, 168-179, 271-275, 346-362).
template <class P>
void apply_observable(std::vector<std::complex<P>> &sv, int n, const Observable &obs) {
    auto apply_term = [&](std::vector<std::complex<P>> &v, const Term &t) {
        for (const auto &f : t.factors) apply_operation(v, n, f.name, f.wires, false, {}, f.matrix);
    };
    if (!obs.is_hamiltonian && obs.terms.size() == 1) {
        apply_term(sv, obs.terms[0]);
        return;
    }
    std::vector<std::complex<P>> buf(sv.size(), 0.0), tmp(sv.size());
    const int64_t N = int64_t(sv.size());
    for (const auto &t : obs.terms) {
        par_copy(tmp, sv);
        apply_term(tmp, t);
        const std::complex<P> c(t.coeff);
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < N; i++) buf[size_t(i)] += c * tmp[size_t(i)];
    }
    sv.swap(buf);
}

// ---------------------------------------------------------------------------
// Adjoint Jacobian (AdjointDiffGPU.hpp:499-596, generator map :58-93,
// scaling factors :96-114, updateJacobian :132-162).
// ---------------------------------------------------------------------------
struct Op {
    std::string name;
    std::vector<int> wires;
    std::vector<double> params;
    bool inverse = false;
    Mat matrix;
};

inline bool generator_scale(const std::string &name, double &s) {
    static const std::map<std::string, double> sc{
        {"RX", -0.5},  {"RY", -0.5},  {"RZ", -0.5},  {"IsingXX", -0.5}, {"IsingYY", -0.5},
        {"IsingZZ", -0.5}, {"PhaseShift", 1.0}, {"CRX", -0.5}, {"CRY", -0.5}, {"CRZ", -0.5},
        {"ControlledPhaseShift", 1.0}, {"SingleExcitation", -0.5},
        {"SingleExcitationMinus", -0.5}, {"SingleExcitationPlus", -0.5},
        {"DoubleExcitation", -0.5}, {"DoubleExcitationMinus", -0.5},
        {"DoubleExcitationPlus", -0.5}, {"MultiRZ", -0.5}};
    auto it = sc.find(name);
    if (it == sc.end()) return false;
    s = it->second;
    return true;
}

// Apply the generator of `name` on wires (GateGenerators.hpp:58-160).
template <class P>
void apply_generator(std::vector<std::complex<P>> &sv, int n, const std::string &name,
                     const std::vector<int> &w) {
    const Mat p11 = {0, 0, 0, 1};
    if (name == "RX") return apply_matrix(sv, n, m_paulix(), {}, {w.back()});
    if (name == "RY") return apply_matrix(sv, n, m_pauliy(), {}, {w.back()});
    if (name == "RZ") return apply_matrix(sv, n, m_pauliz(), {}, {w.back()});
    if (name == "PhaseShift") return apply_matrix(sv, n, p11, {}, {w.back()});
    if (name == "CRX" || name == "CRY" || name == "CRZ") {
        apply_matrix(sv, n, p11, {}, {w.front()});
        const Mat g = name == "CRX" ? m_paulix() : name == "CRY" ? m_pauliy() : m_pauliz();
        return apply_matrix(sv, n, g, {}, {w.back()});
    }
    if (name == "ControlledPhaseShift") {
        Mat m(16, 0.0);
        m[15] = 1.0;
        return apply_matrix(sv, n, m, {}, w);
    }
    if (name == "MultiRZ") return apply_operation(sv, n, "GeneratorMultiRZ", w, false, {}, {});
    return apply_operation(sv, n, "Generator" + name, w, false, {}, {});
}

template <class P>
std::vector<std::vector<double>> adjoint_jacobian(const std::vector<std::complex<P>> &final_state,
                                                  int n, const std::vector<Observable> &obs,
                                                  const std::vector<Op> &ops,
                                                  const std::vector<size_t> &trainable) {
    if (trainable.empty()) throw OracleError("No trainable parameters provided.");
    const size_t K = obs.size();
    std::vector<std::vector<double>> jac(K, std::vector<double>(trainable.size(), 0.0));
    size_t num_param_ops = 0;
    for (const auto &op : ops)
        if (!op.params.empty()) num_param_ops++;
    std::vector<std::complex<P>> lambda, mu;
    par_copy(lambda, final_state);
    std::vector<std::vector<std::complex<P>>> bras(K);
    for (size_t k = 0; k < K; k++) {
        par_copy(bras[k], lambda);
        apply_observable(bras[k], n, obs[k]);
    }
    const int64_t N = int64_t(lambda.size());
    size_t tp_number = trainable.size() - 1;
    size_t cur_param = num_param_ops - 1;
    auto tp_it = trainable.rbegin();
    for (int oi = int(ops.size()) - 1; oi >= 0; oi--) {
        const Op &op = ops[size_t(oi)];
        if (op.params.size() > 1)
            throw OracleError("The operation is not supported using the adjoint differentiation method");
        if (op.name == "QubitStateVector" || op.name == "StatePrep" || op.name == "BasisState")
            continue;
        if (tp_it == trainable.rend()) break;
        // mu = lambda before this operation is undone (needed only for a
        // trainable parameter: mu <- G mu)
        const bool grad = !op.params.empty() && cur_param == *tp_it;
        if (grad) par_copy(mu, lambda);
        apply_operation(lambda, n, op.name, op.wires, !op.inverse, op.params, op.matrix);
        if (!op.params.empty()) {
            if (grad) {
                double s = 0;
                if (!generator_scale(op.name, s))
                    throw OracleError("no generator for " + op.name);
                s *= op.inverse ? -1.0 : 1.0;
                apply_generator(mu, n, op.name, op.wires);
                for (size_t k = 0; k < K; k++) {
                    double im = 0;
                    const auto &bra = bras[k];
#pragma omp parallel for reduction(+ : im) schedule(static)
                    for (int64_t i = 0; i < N; i++)
                        im += (std::conj(cd(bra[size_t(i)])) * cd(mu[size_t(i)])).imag();
                    jac[k][tp_number] = -2.0 * s * im;
                }
                tp_number--;
                ++tp_it;
            }
            cur_param--;
        }
        for (size_t k = 0; k < K; k++)
            apply_operation(bras[k], n, op.name, op.wires, !op.inverse, op.params, op.matrix);
    }
    return jac;
}

// CSR sparse <psi|H|psi> (cusparseSpMV + dotc; StateVectorCudaManaged.hpp:795-922).
template <class P, class I>
double expval_sparse(const std::vector<std::complex<P>> &sv, const I *offsets, int64_t nrows,
                     const I *cols, const cd *vals) {
    double re = 0;
#pragma omp parallel for reduction(+ : re) schedule(static)
    for (int64_t r = 0; r < nrows; r++) {
        cd acc = 0;
        for (I p = offsets[r]; p < offsets[r + 1]; p++) acc += vals[p] * cd(sv[size_t(cols[p])]);
        re += (std::conj(cd(sv[size_t(r)])) * acc).real();
    }
    return re;
}

} // namespace oracle
