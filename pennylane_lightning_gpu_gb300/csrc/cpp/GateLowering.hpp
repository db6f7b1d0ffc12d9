// Lowering of named PennyLane operations to engine primitives, and the
// shared-memory gate-fusion planner.
//
// lower_operation() restates the dispatch of the reference
// StateVectorCudaManaged::applyOperation (StateVectorCudaManaged.hpp:198-247)
// and the per-gate methods it reaches (:320-560, :1179-1305): controls are
// the first ctrl_map[name] wires, Pauli rotations take angle -param/2
// (+param/2 for the adjoint, :1372), named constant gates come from the gate
// cache (cuGateCache.hpp:60-161), and anything else needs an explicit
// matrix.  One deliberate difference: Adjoint(Rot/CRot) applies the inverse
// of Rot(phi, theta, omega); the reference applies getRot(omega, theta, phi)
// daggered (StateVectorCudaManaged.hpp:215-224), which differs when phi != omega.
#pragma once

#include <algorithm>
#include <complex>
#include <map>
#include <string>
#include <unordered_map>
#include <vector>

#include "Error.hpp"
#include "cuGates_host.hpp"

namespace Pennylane::Engine {

using cd = std::complex<double>;

struct GateDesc {
    enum Kind { MATRIX, PAULI_ROT, IDENTITY } kind = IDENTITY;
    std::vector<int> tgts;   // state bits, first = most significant matrix bit
    std::vector<int> ctrls;  // state bits
    std::vector<int> cvals;  // control values (1 in all named gates)
    std::vector<cd> matrix;  // MATRIX: 2^t x 2^t row-major (adjoint already applied)
    double angle = 0;        // PAULI_ROT: exp(i angle P)
    std::string paulis;      // PAULI_ROT: letter per target
};

inline int bit_of(size_t n, size_t wire) { return int(n - 1 - wire); }

inline std::vector<cd> dagger(const std::vector<cd> &m) {
    size_t D = 1;
    while (D * D < m.size()) D++;
    std::vector<cd> r(m.size());
    for (size_t i = 0; i < D; i++)
        for (size_t j = 0; j < D; j++) r[i * D + j] = std::conj(m[j * D + i]);
    return r;
}

template <class CFP_t> inline std::vector<cd> to_cd(const std::vector<CFP_t> &m) {
    std::vector<cd> r(m.size());
    for (size_t i = 0; i < m.size(); i++) r[i] = cd(double(m[i].x), double(m[i].y));
    return r;
}

inline const std::unordered_map<std::string, size_t> &ctrl_map() {
    static const std::unordered_map<std::string, size_t> m{
        {"Identity", 0}, {"PauliX", 0}, {"PauliY", 0}, {"PauliZ", 0}, {"Hadamard", 0}, {"T", 0},
        {"S", 0},        {"RX", 0},     {"RY", 0},     {"RZ", 0},     {"Rot", 0},      {"PhaseShift", 0},
        {"ControlledPhaseShift", 1},    {"CNOT", 1},   {"SWAP", 0},   {"CY", 1},       {"CZ", 1},
        {"CRX", 1},      {"CRY", 1},    {"CRZ", 1},    {"CRot", 1},   {"CSWAP", 1},    {"Toffoli", 2}};
    return m;
}

// Named constant gates (value of the reference's pre-populated gate cache).
inline bool constant_gate(const std::string &name, std::vector<cd> &m) {
    using C = cuDoubleComplex;
    namespace G = Pennylane::CUDA::cuGates;
    if (name == "PauliX" || name == "CNOT" || name == "Toffoli") m = to_cd(G::getPauliX<C>());
    else if (name == "PauliY" || name == "CY") m = to_cd(G::getPauliY<C>());
    else if (name == "PauliZ" || name == "CZ") m = to_cd(G::getPauliZ<C>());
    else if (name == "Hadamard") m = to_cd(G::getHadamard<C>());
    else if (name == "S") m = to_cd(G::getS<C>());
    else if (name == "T") m = to_cd(G::getT<C>());
    else if (name == "SWAP" || name == "CSWAP") m = to_cd(G::getSWAP<C>());
    else if (name == "Identity" || name == "I") m = to_cd(G::getIdentity<C>());
    else return false;
    return true;
}

// Generator matrices on the op's own bit order [ctrls..., tgts...]
// (AdjointDiffGPU.hpp:58-114 + GateGenerators.hpp:58-322), and scale factors.
inline bool generator_of(const std::string &name, size_t nbits, std::vector<cd> &g, double &scale) {
    using C = cuDoubleComplex;
    namespace G = Pennylane::CUDA::cuGates;
    const std::vector<cd> X = to_cd(G::getPauliX<C>()), Y = to_cd(G::getPauliY<C>()), Z = to_cd(G::getPauliZ<C>());
    auto kron = [](const std::vector<cd> &a, const std::vector<cd> &b) {
        size_t da = 1, db = 1;
        while (da * da < a.size()) da++;
        while (db * db < b.size()) db++;
        std::vector<cd> m(da * db * da * db);
        for (size_t i = 0; i < da; i++)
            for (size_t j = 0; j < da; j++)
                for (size_t k = 0; k < db; k++)
                    for (size_t l = 0; l < db; l++) m[(i * db + k) * (da * db) + (j * db + l)] = a[i * da + j] * b[k * db + l];
        return m;
    };
    const std::vector<cd> P11 = {0, 0, 0, 1};
    scale = -0.5;
    if (name == "RX") g = X;
    else if (name == "RY") g = Y;
    else if (name == "RZ") g = Z;
    else if (name == "PhaseShift") { g = P11; scale = 1.0; }
    else if (name == "CRX") g = kron(P11, X);
    else if (name == "CRY") g = kron(P11, Y);
    else if (name == "CRZ") g = kron(P11, Z);
    else if (name == "ControlledPhaseShift") { g = kron(P11, P11); scale = 1.0; }
    else if (name == "IsingXX") g = kron(X, X);
    else if (name == "IsingYY") g = kron(Y, Y);
    else if (name == "IsingZZ") g = kron(Z, Z);
    else if (name == "SingleExcitation") g = to_cd(G::getGeneratorSingleExcitation<C>());
    else if (name == "SingleExcitationMinus") g = to_cd(G::getGeneratorSingleExcitationMinus<C>());
    else if (name == "SingleExcitationPlus") g = to_cd(G::getGeneratorSingleExcitationPlus<C>());
    else if (name == "DoubleExcitation") g = to_cd(G::getGeneratorDoubleExcitation<C>());
    else if (name == "DoubleExcitationMinus") g = to_cd(G::getGeneratorDoubleExcitationMinus<C>());
    else if (name == "DoubleExcitationPlus") g = to_cd(G::getGeneratorDoubleExcitationPlus<C>());
    else if (name == "MultiRZ") {
        if (nbits > 6) return false;
        g = Z;
        for (size_t k = 1; k < nbits; k++) g = kron(g, Z);
    } else
        return false;
    return true;
}

inline bool has_generator(const std::string &name) {
    static const char *names[] = {"RX", "RY", "RZ", "PhaseShift", "CRX", "CRY", "CRZ", "ControlledPhaseShift",
                                  "IsingXX", "IsingYY", "IsingZZ", "SingleExcitation", "SingleExcitationMinus",
                                  "SingleExcitationPlus", "DoubleExcitation", "DoubleExcitationMinus",
                                  "DoubleExcitationPlus", "MultiRZ"};
    for (const char *s : names)
        if (name == s) return true;
    return false;
}

// user_matrix: the optional gate_matrix of applyOperation (PennyLane order).
inline GateDesc lower_operation(size_t n, const std::string &name, const std::vector<size_t> &wires, bool adjoint,
                                const std::vector<double> &params, const std::vector<cd> &user_matrix) {
    using C = cuDoubleComplex;
    namespace G = Pennylane::CUDA::cuGates;
    for (size_t w : wires) PL_ABORT_IF(w >= n, "Wire index out of range");
    GateDesc d;
    const auto it = ctrl_map().find(name);
    const size_t nc = it == ctrl_map().end() ? 0 : it->second;
    PL_ABORT_IF(wires.size() < nc, "Not enough wires for the operation");
    auto P = [&](size_t i) {
        PL_ABORT_IF(params.size() <= i, "Missing parameter for the operation");
        return params[i];
    };
    auto set_wires = [&](size_t ncontrols) {
        d.ctrls.clear();
        d.tgts.clear();
        d.cvals.clear();
        for (size_t k = 0; k < wires.size(); k++) {
            if (k < ncontrols) {
                d.ctrls.push_back(bit_of(n, wires[k]));
                d.cvals.push_back(1);
            } else {
                d.tgts.push_back(bit_of(n, wires[k]));
            }
        }
    };
    auto mat = [&](std::vector<cd> m, size_t ncontrols) {
        d.kind = GateDesc::MATRIX;
        d.matrix = adjoint ? dagger(m) : std::move(m);
        set_wires(ncontrols);
    };
    if (name == "Identity" || name == "I") {
        d.kind = GateDesc::IDENTITY;
        return d;
    }
    if (name == "RX" || name == "RY" || name == "RZ" || name == "CRX" || name == "CRY" || name == "CRZ") {
        // exp(-i*theta/2*P) as an explicit 2x2 matrix (adjoint: theta -> -theta)
        const double th = adjoint ? -P(0) : P(0);
        const char p = name.back();
        std::vector<cd> m = p == 'X' ? to_cd(G::getRX<C>(th)) : p == 'Y' ? to_cd(G::getRY<C>(th)) : to_cd(G::getRZ<C>(th));
        d.kind = GateDesc::MATRIX;
        d.matrix = m;
        set_wires(nc);
        return d;
    }
    if (name == "Rot" || name == "CRot") {
        mat(to_cd(G::getRot<C>(P(0), P(1), P(2))), nc);
        return d;
    }
    if (name == "PhaseShift" || name == "ControlledPhaseShift") {
        PL_ABORT_IF(wires.empty(), "PhaseShift needs a wire");
        mat(to_cd(G::getPhaseShift<C>(P(0))), wires.size() - 1);
        return d;
    }
    if (name == "MultiRZ" || name == "IsingXX" || name == "IsingYY" || name == "IsingZZ") {
        d.kind = GateDesc::PAULI_ROT;
        d.angle = adjoint ? P(0) / 2 : -P(0) / 2;
        d.paulis = std::string(wires.size(), name == "MultiRZ" ? 'Z' : name.back());
        set_wires(0);
        return d;
    }
    if (name == "SingleExcitation") { mat(to_cd(G::getSingleExcitation<C>(P(0))), 0); return d; }
    if (name == "SingleExcitationMinus") { mat(to_cd(G::getSingleExcitationMinus<C>(P(0))), 0); return d; }
    if (name == "SingleExcitationPlus") { mat(to_cd(G::getSingleExcitationPlus<C>(P(0))), 0); return d; }
    if (name == "DoubleExcitation") { mat(to_cd(G::getDoubleExcitation<C>(P(0))), 0); return d; }
    if (name == "DoubleExcitationMinus") { mat(to_cd(G::getDoubleExcitationMinus<C>(P(0))), 0); return d; }
    if (name == "DoubleExcitationPlus") { mat(to_cd(G::getDoubleExcitationPlus<C>(P(0))), 0); return d; }
    std::vector<cd> m;
    if (constant_gate(name, m)) {
        mat(m, nc);
        return d;
    }
    PL_ABORT_IF(user_matrix.empty(), ("Currently unsupported gate: " + name).c_str());
    mat(user_matrix, nc);
    return d;
}

// Dense matrix of a primitive over the bit list [ctrls..., tgts...] with the
// controls folded in (used by the fused adjoint step).  Returns false when the
// operation spans more than `max_bits` bits.
inline bool dense_on_bits(const GateDesc &d, std::vector<int> &bits, std::vector<cd> &out, size_t max_bits = 4) {
    bits = d.ctrls;
    bits.insert(bits.end(), d.tgts.begin(), d.tgts.end());
    if (bits.empty() || bits.size() > max_bits) return false;
    const size_t c = d.ctrls.size(), t = d.tgts.size();
    const size_t Dt = size_t(1) << t, D = size_t(1) << (c + t);
    std::vector<cd> u(Dt * Dt);
    if (d.kind == GateDesc::MATRIX) {
        u = d.matrix;
    } else if (d.kind == GateDesc::PAULI_ROT) {
        // exp(i angle P) = cos(angle) I + i sin(angle) P
        const cd I1(0, 1);
        std::vector<cd> Pm(Dt * Dt, 0.0);
        for (size_t col = 0; col < Dt; col++) {
            // P|col>: letters act on matrix bits, tgts[0] = MSB
            size_t row = col;
            cd amp = 1.0;
            for (size_t k = 0; k < t; k++) {
                const size_t b = t - 1 - k;
                const int v = int((col >> b) & 1);
                switch (d.paulis[k]) {
                case 'X': row ^= size_t(1) << b; break;
                case 'Y': row ^= size_t(1) << b; amp *= v ? -I1 : I1; break;
                case 'Z': amp *= v ? -1.0 : 1.0; break;
                default: break;
                }
            }
            Pm[row * Dt + col] = amp;
        }
        for (size_t i = 0; i < Dt * Dt; i++) u[i] = I1 * std::sin(d.angle) * Pm[i];
        for (size_t i = 0; i < Dt; i++) u[i * Dt + i] += std::cos(d.angle);
    } else {
        return false;
    }
    out.assign(D * D, 0.0);
    size_t cidx = 0;  // index of the control block (ctrl values as MSBs)
    for (size_t k = 0; k < c; k++) cidx = (cidx << 1) | size_t(d.cvals[k] ? 1 : 0);
    for (size_t blk = 0; blk < (size_t(1) << c); blk++) {
        for (size_t r = 0; r < Dt; r++)
            for (size_t col = 0; col < Dt; col++) {
                const size_t R = blk * Dt + r, Cc = blk * Dt + col;
                out[R * D + Cc] = (blk == cidx) ? u[r * Dt + col] : (r == col ? cd(1.0) : cd(0.0));
            }
    }
    return true;
}

// ---------------------------------------------------------------------------
// Fusion planner: greedy blocks of 1/2-target matrix gates whose targets fit a
// tile of `kmax` bits made of the low run 0..m-1 (m >= mmin) plus at most
// `max_hi` higher bits.
// A gate may join the current block only if it commutes with every gate the
// scan has skipped so far (its bits are disjoint from theirs).
// ---------------------------------------------------------------------------
struct FusedBlock {
    std::vector<int> tile_bits;        // empty: apply `single` directly
    std::vector<size_t> gates;         // indices into the input list
};

inline bool tile_for(const std::vector<int> &gate_bits, int kmax, int mmin, size_t n, std::vector<int> &tile,
                     size_t max_hi = 6) {
    for (int m = std::min<int>(kmax, int(n)); m >= std::min<int>(mmin, int(n)); m--) {
        std::vector<int> hi;
        for (int b : gate_bits)
            if (b >= m) hi.push_back(b);
        std::sort(hi.begin(), hi.end());
        hi.erase(std::unique(hi.begin(), hi.end()), hi.end());
        if (int(hi.size()) <= kmax - m && hi.size() <= max_hi) {
            tile.clear();
            for (int b = 0; b < m; b++) tile.push_back(b);
            tile.insert(tile.end(), hi.begin(), hi.end());
            return true;
        }
    }
    return false;
}

inline bool fusable(const GateDesc &d) {
    return d.kind == GateDesc::MATRIX && (d.tgts.size() == 1 || d.tgts.size() == 2) && d.ctrls.size() <= 4;
}

// Fold each uncontrolled 1-target matrix gate into the previous one on the
// same bit when no gate touching that bit lies between them (the gates in
// between act on other bits and commute with both): the earlier gate becomes
// the 2x2 product and the later one IDENTITY.  One dense body costs no more
// arithmetic than the structured bodies it replaces (complex128: 12 FP64
// operations per pair either way for RX.RY.RZ) and saves their shared-memory
// round trips.
inline void merge_1q_runs(std::vector<GateDesc> &gates) {
    std::unordered_map<int, size_t> pending;  // bit -> index of the gate that absorbs the next one
    for (size_t i = 0; i < gates.size(); i++) {
        GateDesc &g = gates[i];
        if (g.kind == GateDesc::IDENTITY) continue;
        if (g.kind == GateDesc::MATRIX && g.tgts.size() == 1 && g.ctrls.empty() && g.matrix.size() == 4) {
            const auto it = pending.find(g.tgts[0]);
            if (it != pending.end()) {
                GateDesc &a = gates[it->second];
                const std::vector<cd> &b = g.matrix;
                const std::vector<cd> m = a.matrix;
                a.matrix = {b[0] * m[0] + b[1] * m[2], b[0] * m[1] + b[1] * m[3], b[2] * m[0] + b[3] * m[2],
                            b[2] * m[1] + b[3] * m[3]};
                g = GateDesc{};
                continue;
            }
            pending[g.tgts[0]] = i;
            continue;
        }
        for (int b : g.tgts) pending.erase(b);
        for (int b : g.ctrls) pending.erase(b);
    }
}

inline std::vector<FusedBlock> plan_fusion(const std::vector<GateDesc> &gates, size_t n, int kmax, int mmin,
                                           size_t min_block = 2, size_t max_hi = 6) {
    std::vector<FusedBlock> out;
    std::vector<char> done(gates.size(), 0);
    size_t first = 0;
    while (first < gates.size()) {
        while (first < gates.size() && done[first]) first++;
        if (first >= gates.size()) break;
        FusedBlock blk;
        std::vector<int> bits;
        uint64_t blocked = 0;
        std::vector<int> tile;
        for (size_t i = first; i < gates.size(); i++) {
            if (done[i]) continue;
            const GateDesc &g = gates[i];
            uint64_t wmask = 0;
            for (int b : g.tgts) wmask |= uint64_t(1) << b;
            for (int b : g.ctrls) wmask |= uint64_t(1) << b;
            if (g.kind == GateDesc::IDENTITY) {
                if (!(wmask & blocked)) {
                    blk.gates.push_back(i);
                }
                continue;
            }
            if (wmask & blocked) {
                blocked |= wmask;
                continue;
            }
            bool ok = false;
            if (fusable(g)) {
                std::vector<int> trial(bits);
                trial.insert(trial.end(), g.tgts.begin(), g.tgts.end());
                std::vector<int> t2;
                if (tile_for(trial, kmax, mmin, n, t2, max_hi)) {
                    ok = true;
                    bits = trial;
                    tile = t2;
                }
            }
            if (ok) {
                blk.gates.push_back(i);
            } else {
                blocked |= wmask;
                if (blk.gates.empty()) break;  // first gate cannot be fused: emit alone
            }
        }
        size_t nreal = 0;
        for (size_t gi : blk.gates)
            if (gates[gi].kind != GateDesc::IDENTITY) nreal++;
        if (nreal >= min_block) {
            blk.tile_bits = tile;
            for (size_t gi : blk.gates) done[gi] = 1;
            out.push_back(blk);
        } else {
            // emit the first pending gate on its own
            FusedBlock single;
            single.gates.push_back(first);
            done[first] = 1;
            out.push_back(single);
        }
    }
    return out;
}

} // namespace Pennylane::Engine
