// Host test of the engine's gate lowering (GateLowering.hpp::lower_operation
// and the cuGates_host.hpp factories it uses) against the oracle
// (oracle/sv_oracle.hpp::apply_operation): for every named operation, with
// and without the adjoint flag, random parameters and random wires on 5
// qubits, the operator built column by column from the lowered primitive
// equals the oracle's within 1e-12.  User matrices (QubitUnitary on 2 and 3
// wires) are checked the same way.
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdio>
#include <random>
#include <string>
#include <vector>

#include "desc_apply.hpp"
#include "sv_oracle.hpp"

using namespace Pennylane::Engine;
using hosttest::apply_desc;
using hosttest::cdv;

static long bad = 0;

static void fail(const char *what, const std::string &name, double v) {
    if (bad < 20) std::printf("bad %s (%s): %g\n", what, name.c_str(), v);
    bad++;
}

int main() {
    struct Spec {
        const char *name;
        int nwires, nparams;
    };
    const Spec specs[] = {
        {"Identity", 1, 0}, {"PauliX", 1, 0}, {"PauliY", 1, 0}, {"PauliZ", 1, 0}, {"Hadamard", 1, 0}, {"S", 1, 0},
        {"T", 1, 0}, {"RX", 1, 1}, {"RY", 1, 1}, {"RZ", 1, 1}, {"Rot", 1, 3}, {"PhaseShift", 1, 1},
        {"CNOT", 2, 0}, {"CY", 2, 0}, {"CZ", 2, 0}, {"SWAP", 2, 0}, {"CRX", 2, 1}, {"CRY", 2, 1}, {"CRZ", 2, 1},
        {"CRot", 2, 3}, {"ControlledPhaseShift", 2, 1}, {"IsingXX", 2, 1}, {"IsingYY", 2, 1}, {"IsingZZ", 2, 1},
        {"SingleExcitation", 2, 1}, {"SingleExcitationMinus", 2, 1}, {"SingleExcitationPlus", 2, 1},
        {"CSWAP", 3, 0}, {"Toffoli", 3, 0}, {"MultiRZ", 1, 1}, {"MultiRZ", 3, 1}, {"MultiRZ", 5, 1},
        {"DoubleExcitation", 4, 1}, {"DoubleExcitationMinus", 4, 1}, {"DoubleExcitationPlus", 4, 1}};
    const int n = 5;
    const size_t N = size_t(1) << n;
    std::mt19937 gen(11);
    std::uniform_real_distribution<double> ang(-3.1, 3.1);
    std::normal_distribution<double> nd;
    long nchecks = 0;
    for (const Spec &sp : specs) {
        for (int rep = 0; rep < 6; rep++) {
            for (bool adj : {false, true}) {
                std::vector<size_t> w;
                while (int(w.size()) < sp.nwires) {
                    const size_t x = gen() % size_t(n);
                    if (std::find(w.begin(), w.end(), x) == w.end()) w.push_back(x);
                }
                std::vector<double> p;
                for (int k = 0; k < sp.nparams; k++) p.push_back(ang(gen));
                const GateDesc d = lower_operation(size_t(n), sp.name, w, adj, p, {});
                const std::vector<int> wi(w.begin(), w.end());
                double err = 0;
                for (size_t col = 0; col < N; col++) {
                    cdv e(N, 0.0), o(N, 0.0);
                    e[col] = o[col] = 1.0;
                    if (!apply_desc(e, d)) fail("not expandable", sp.name, 0);
                    oracle::apply_operation<double>(o, n, sp.name, wi, adj, p, {});
                    for (size_t r = 0; r < N; r++) err = std::max(err, std::abs(e[r] - o[r]));
                }
                nchecks++;
                if (err > 1e-12) fail("operator differs from the oracle", sp.name, err);
            }
        }
    }
    // a user matrix on 2 and 3 wires (PennyLane order: wires[0] most significant)
    for (int t : {2, 3}) {
        const size_t D = size_t(1) << t;
        cdv m(D * D);
        for (auto &x : m) x = {nd(gen), nd(gen)};
        std::vector<size_t> w;
        while (w.size() < size_t(t)) {
            const size_t x = gen() % size_t(n);
            if (std::find(w.begin(), w.end(), x) == w.end()) w.push_back(x);
        }
        for (bool adj : {false, true}) {
            const GateDesc d = lower_operation(size_t(n), "QubitUnitary", w, adj, {}, m);
            const std::vector<int> wi(w.begin(), w.end());
            double err = 0;
            for (size_t col = 0; col < N; col++) {
                cdv e(N, 0.0), o(N, 0.0);
                e[col] = o[col] = 1.0;
                apply_desc(e, d);
                oracle::apply_operation<double>(o, n, "QubitUnitary", wi, adj, {}, oracle::Mat(m.begin(), m.end()));
                for (size_t r = 0; r < N; r++) err = std::max(err, std::abs(e[r] - o[r]));
            }
            nchecks++;
            if (err > 1e-12) fail("user matrix differs from the oracle", "QubitUnitary", err);
        }
    }
    std::printf("operators %ld bad %ld\n", nchecks, bad);
    return bad == 0 ? 0 : 1;
}
