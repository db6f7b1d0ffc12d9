// Host test of the register-group split of a fused gate block
// (lgpu_fused_plan.h::group_fused_gates), which reorders a launch's gates:
// random blocks of 1- and 2-target gates with in-tile controls on tiles of
// 6..12 positions, grouped for 2, 3 and 4 register positions.  Checks:
//  * the groups cover the permuted gate list contiguously, every gate once,
//    with its per-gate constants permuted alongside;
//  * a register group lists R ascending tile positions that hold every
//    position its gates touch, and each gate's local target and local
//    control mask and values match its tile fields; other groups hold one
//    gate;
//  * applying the gates in group order gives the state of the original
//    order within 1e-12 (random unitaries on a random tile state).
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdio>
#include <random>
#include <vector>

#include "lgpu_fused_plan.h"

using lgpu::FGate;
using lgpu::FGroup;
using cd = std::complex<double>;

struct KC {
    int id;
    int pad[3];
};

static long bad = 0;

static void fail(const char *what, int trial, long v) {
    if (bad < 20) std::printf("bad %s (trial %d): %ld\n", what, trial, v);
    bad++;
}

static std::vector<cd> random_unitary(int d, std::mt19937 &gen) {
    std::normal_distribution<double> nd;
    std::vector<cd> m(size_t(d * d));
    for (auto &x : m) x = cd(nd(gen), nd(gen));
    // Gram-Schmidt on the columns
    for (int c = 0; c < d; c++) {
        for (int p = 0; p < c; p++) {
            cd dot = 0;
            for (int r = 0; r < d; r++) dot += std::conj(m[size_t(r * d + p)]) * m[size_t(r * d + c)];
            for (int r = 0; r < d; r++) m[size_t(r * d + c)] -= dot * m[size_t(r * d + p)];
        }
        double nrm = 0;
        for (int r = 0; r < d; r++) nrm += std::norm(m[size_t(r * d + c)]);
        nrm = std::sqrt(nrm);
        for (int r = 0; r < d; r++) m[size_t(r * d + c)] /= nrm;
    }
    return m;
}

static void apply(std::vector<cd> &t, const FGate &g, const std::vector<cd> &m) {
    const uint32_t E = uint32_t(t.size());
    const uint32_t tm = (1u << g.q0) | (g.ntgt == 2 ? (1u << g.q1) : 0u);
    for (uint32_t i = 0; i < E; i++) {
        if ((i & tm) || (i & g.in_mask) != g.in_val) continue;
        if (g.ntgt == 1) {
            const uint32_t j = i | (1u << g.q0);
            const cd a = t[i], b = t[j];
            t[i] = m[0] * a + m[1] * b;
            t[j] = m[2] * a + m[3] * b;
        } else {
            const uint32_t idx[4] = {i, i | (1u << g.q1), i | (1u << g.q0), i | (1u << g.q0) | (1u << g.q1)};
            cd a[4], y[4];
            for (int c = 0; c < 4; c++) a[c] = t[idx[c]];
            for (int r = 0; r < 4; r++) {
                y[r] = 0;
                for (int c = 0; c < 4; c++) y[r] += m[size_t(r * 4 + c)] * a[c];
            }
            for (int r = 0; r < 4; r++) t[idx[r]] = y[r];
        }
    }
}

int main() {
    std::mt19937 gen(99);
    std::normal_distribution<double> nd;
    long ngroups_total = 0, nreg = 0, ngates = 0;
    int trial = 0;
    for (int k = 6; k <= 12; k++) {
        for (int R = 2; R <= 4; R++) {
            for (int rep = 0; rep < 60; rep++, trial++) {
                const int cnt = 1 + int(gen() % lgpu::kFusedMaxGates);
                std::vector<FGate> g(static_cast<size_t>(cnt));
                std::vector<KC> kc(static_cast<size_t>(cnt));
                std::vector<std::vector<cd>> mats(static_cast<size_t>(cnt));
                // a few hot positions make groups likely
                const int hot = 2 + int(gen() % 4);
                auto pos = [&]() { return int(gen() % 3 ? gen() % uint32_t(hot) : gen() % uint32_t(k)); };
                for (int i = 0; i < cnt; i++) {
                    FGate x{};
                    x.ntgt = uint8_t(gen() % 6 == 0 ? 2 : 1);
                    x.q0 = uint8_t(pos());
                    if (x.ntgt == 2)
                        do x.q1 = uint8_t(pos()); while (x.q1 == x.q0);
                    const int nctrl = int(gen() % 3);
                    for (int c = 0; c < nctrl; c++) {
                        const int q = pos();
                        if (q == x.q0 || (x.ntgt == 2 && q == x.q1)) continue;
                        x.in_mask |= 1u << q;
                        if (gen() % 3) x.in_val |= 1u << q;
                    }
                    x.in_val &= x.in_mask;
                    x.mat_off = uint32_t(i);  // the gate's identity
                    g[size_t(i)] = x;
                    kc[size_t(i)].id = i;
                    mats[size_t(i)] = random_unitary(x.ntgt == 2 ? 4 : 2, gen);
                }
                const std::vector<FGate> orig = g;
                std::vector<FGroup> groups(static_cast<size_t>(cnt));
                const int ng = lgpu::group_fused_gates(g.data(), kc.data(), cnt, k, R, groups.data());
                ngroups_total += ng;
                ngates += cnt;
                // coverage and permutation
                std::vector<int> seen(static_cast<size_t>(cnt), 0);
                int next = 0;
                for (int q = 0; q < ng; q++) {
                    const FGroup &G = groups[size_t(q)];
                    if (G.first != next) fail("groups not contiguous", trial, G.first);
                    next = G.first + G.count;
                    if (G.kind == 1 && G.count != 1) fail("single group with several gates", trial, G.count);
                    if (G.kind == 0) {
                        nreg++;
                        uint32_t set = 0;
                        for (int b = 0; b < R; b++) {
                            if (G.p[b] >= k) fail("group position outside the tile", trial, G.p[b]);
                            if (b > 0 && G.p[b] <= G.p[b - 1]) fail("group positions not ascending", trial, b);
                            set |= 1u << G.p[b];
                        }
                        for (int t = G.first; t < G.first + G.count; t++) {
                            const FGate &x = g[size_t(t)];
                            if (x.ntgt != 1) fail("2-target gate in a register group", trial, t);
                            if (((x.in_mask | (1u << x.q0)) & ~set) != 0) fail("gate outside its group", trial, t);
                            if (x.lt >= R || G.p[x.lt] != x.q0) fail("local target", trial, t);
                            uint32_t lcm = 0, lcv = 0;
                            for (int b = 0; b < R; b++) {
                                if ((x.in_mask >> G.p[b]) & 1u) lcm |= 1u << b;
                                if ((x.in_val >> G.p[b]) & 1u) lcv |= 1u << b;
                            }
                            if (lcm != x.lcm || lcv != x.lcv) fail("local controls", trial, t);
                        }
                    }
                }
                if (next != cnt) fail("groups do not cover the gates", trial, next);
                for (int i = 0; i < cnt; i++) {
                    const int id = int(g[size_t(i)].mat_off);
                    if (id < 0 || id >= cnt) {
                        fail("gate identity", trial, id);
                        continue;
                    }
                    seen[size_t(id)]++;
                    if (kc[size_t(i)].id != id) fail("constants not permuted with their gate", trial, i);
                    const FGate &o = orig[size_t(id)];
                    if (o.q0 != g[size_t(i)].q0 || o.in_mask != g[size_t(i)].in_mask || o.ntgt != g[size_t(i)].ntgt)
                        fail("gate fields changed", trial, i);
                }
                for (int i = 0; i < cnt; i++)
                    if (seen[size_t(i)] != 1) fail("gate not placed exactly once", trial, i);
                // semantics
                std::vector<cd> a(size_t(1) << k);
                for (auto &x : a) x = cd(nd(gen), nd(gen));
                std::vector<cd> b = a;
                for (int i = 0; i < cnt; i++) apply(a, orig[size_t(i)], mats[size_t(i)]);
                for (int i = 0; i < cnt; i++) apply(b, g[size_t(i)], mats[g[size_t(i)].mat_off]);
                double err = 0;
                for (size_t i = 0; i < a.size(); i++) err = std::max(err, std::abs(a[i] - b[i]));
                if (err > 1e-12) fail("group order changes the state", trial, long(err * 1e12));
            }
        }
    }
    std::printf("blocks %d gates %ld groups %ld register groups %ld bad %ld\n", trial, ngates, ngroups_total, nreg,
                bad);
    return bad == 0 ? 0 : 1;
}
