// Host test of the gate lowering and the fusion planner (GateLowering.hpp).
// Random circuits of named gates on 5..10 qubits are lowered the way
// StateVectorCudaManaged::applyDescs lowers them (1- and 2-target Pauli
// rotations become matrices), merged (merge_1q_runs) and planned
// (plan_fusion) for several tile shapes.  Checks:
//  * every lowered gate lands in exactly one block;
//  * a fused block holds at least min_block gates, only 1- and 2-target
//    matrix gates with at most 4 controls, and a tile of at most kmax bits
//    made of the low run 0..m-1 (m >= min(mmin, n)) plus at most max_hi
//    higher bits that contains every target;
//  * applying the blocks in plan order (gates of a block in listed order)
//    gives the state of the unmerged gates applied one by one, within 1e-12.
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdio>
#include <random>
#include <string>
#include <vector>

#include "desc_apply.hpp"

using namespace Pennylane::Engine;
using hosttest::apply_desc;
using hosttest::cdv;

static long bad = 0;

static void fail(const char *what, int trial, double v) {
    if (bad < 20) std::printf("bad %s (trial %d): %g\n", what, trial, v);
    bad++;
}

struct Spec {
    const char *name;
    int nwires, nparams;
};

int main() {
    const Spec specs[] = {{"PauliX", 1, 0},   {"PauliY", 1, 0},     {"PauliZ", 1, 0},
                          {"Hadamard", 1, 0}, {"S", 1, 0},          {"T", 1, 0},
                          {"RX", 1, 1},       {"RY", 1, 1},         {"RZ", 1, 1},
                          {"Rot", 1, 3},      {"PhaseShift", 1, 1}, {"CNOT", 2, 0},
                          {"CZ", 2, 0},       {"CY", 2, 0},         {"SWAP", 2, 0},
                          {"CRX", 2, 1},      {"CRY", 2, 1},        {"CRZ", 2, 1},
                          {"CRot", 2, 3},     {"ControlledPhaseShift", 2, 1},
                          {"IsingXX", 2, 1},  {"IsingYY", 2, 1},    {"IsingZZ", 2, 1},
                          {"SingleExcitation", 2, 1},               {"Toffoli", 3, 0},
                          {"CSWAP", 3, 0},    {"MultiRZ", 3, 1},    {"DoubleExcitation", 4, 1},
                          {"Identity", 1, 0}};
    const int nspecs = int(sizeof(specs) / sizeof(specs[0]));
    struct Shape {
        int kmax, mmin;
        size_t max_hi;
    };
    const Shape shapes[] = {{4, 2, 2}, {5, 3, 2}, {6, 3, 3}, {8, 5, 3}, {10, 5, 8}};
    std::mt19937 gen(2024);
    std::uniform_real_distribution<double> ang(-3.1, 3.1), nrm(-1.0, 1.0);
    long nblocks = 0, nfused = 0, ngates = 0;
    int trial = 0;
    for (int n = 5; n <= 10; n++) {
        for (int rep = 0; rep < 40; rep++, trial++) {
            // random circuit, biased towards 1-qubit rotations (merge candidates)
            std::vector<GateDesc> descs;
            const int len = 20 + int(gen() % 40);
            for (int g = 0; g < len; g++) {
                const Spec &sp = (gen() % 3 == 0) ? specs[6 + gen() % 4] : specs[gen() % nspecs];
                if (sp.nwires > n) continue;
                std::vector<size_t> w;
                while (int(w.size()) < sp.nwires) {
                    const size_t x = gen() % size_t(n);
                    if (std::find(w.begin(), w.end(), x) == w.end()) w.push_back(x);
                }
                std::vector<double> p;
                for (int k = 0; k < sp.nparams; k++) p.push_back(ang(gen));
                GateDesc d = lower_operation(size_t(n), sp.name, w, gen() % 4 == 0, p, {});
                if (d.kind == GateDesc::PAULI_ROT && d.tgts.size() <= 2 && d.ctrls.empty()) {
                    std::vector<int> bits;
                    cdv m;
                    if (dense_on_bits(d, bits, m, 2)) {
                        d.kind = GateDesc::MATRIX;
                        d.matrix = m;
                    }
                }
                descs.push_back(d);
            }
            ngates += long(descs.size());
            cdv psi(size_t(1) << n);
            for (auto &x : psi) x = {nrm(gen), nrm(gen)};
            cdv ref = psi;
            for (const auto &d : descs)
                if (!apply_desc(ref, d)) fail("gate not expandable", trial, 0);
            std::vector<GateDesc> merged = descs;
            merge_1q_runs(merged);
            for (const Shape &sh : shapes) {
                const int kmax = std::min(sh.kmax, n), mmin = std::min(sh.mmin, kmax);
                const auto plan = plan_fusion(merged, size_t(n), kmax, mmin, 2, sh.max_hi);
                std::vector<int> seen(merged.size(), 0);
                cdv out = psi;
                for (const auto &blk : plan) {
                    nblocks++;
                    for (size_t gi : blk.gates) {
                        if (gi >= merged.size()) {
                            fail("gate index out of range", trial, double(gi));
                            continue;
                        }
                        seen[gi]++;
                        if (!apply_desc(out, merged[gi])) fail("gate not expandable", trial, double(gi));
                    }
                    if (blk.tile_bits.empty()) {
                        if (blk.gates.size() != 1) fail("single block with several gates", trial, blk.gates.size());
                        continue;
                    }
                    nfused++;
                    const auto &tb = blk.tile_bits;
                    int m = 0;
                    while (m < int(tb.size()) && tb[size_t(m)] == m) m++;
                    if (int(tb.size()) > kmax) fail("tile larger than kmax", trial, double(tb.size()));
                    if (m < mmin) fail("low run shorter than mmin", trial, double(m));
                    if (tb.size() - size_t(m) > sh.max_hi) fail("too many high bits", trial, double(tb.size() - m));
                    size_t nreal = 0;
                    for (size_t gi : blk.gates) {
                        const GateDesc &d = merged[gi];
                        if (d.kind == GateDesc::IDENTITY) continue;
                        nreal++;
                        if (!fusable(d)) fail("non-fusable gate in a fused block", trial, double(gi));
                        for (int b : d.tgts)
                            if (std::find(tb.begin(), tb.end(), b) == tb.end()) fail("target outside the tile", trial, b);
                    }
                    if (nreal < 2) fail("fused block with fewer than 2 gates", trial, double(nreal));
                }
                for (size_t i = 0; i < merged.size(); i++)
                    if (seen[i] != 1) fail("gate not planned exactly once", trial, double(seen[i]));
                double err = 0;
                for (size_t i = 0; i < out.size(); i++) err = std::max(err, std::abs(out[i] - ref[i]));
                if (err > 1e-12) fail("plan changes the state", trial, err);
            }
        }
    }
    std::printf("circuits %d gates %ld blocks %ld fused %ld bad %ld\n", trial, ngates, nblocks, nfused, bad);
    return bad == 0 ? 0 : 1;
}
