// Records of a fused gate block (one launch of the shared-memory tile
// kernel) and the host-side split of its gates into register groups.  Plain
// C++ (no CUDA types), so the grouping can be unit-tested on the host.
#pragma once

#include <algorithm>
#include <complex>
#include <cstdint>
#include <cstring>
#include <vector>

#include "lgpu.h"

namespace lgpu {

constexpr int kFusedMaxGates = 96;
constexpr int kDiagTableBits = 4;  // phase tables of folded diagonal gates: at most 4 tile positions
constexpr int kDiagTableMark = 3;  // gate record ntgt of a folded phase table
constexpr int kFusedMatPool = 2304;  // matrix elements, in the state's precision

struct FGate {
    uint8_t ntgt, q0, q1, body;  // q0 = most significant matrix bit; body: Body1 of a 1-target gate
    uint8_t lt, lcm, lcv, pad;   // register group: local target, local control mask and values;
                                 // pad = 1: diag(+-1, +-1) (complex128 float-float sign flips)
    uint32_t in_mask, in_val;    // controls inside the tile (tile positions)
    uint32_t mat_off;            // into the matrix pool
    uint64_t out_mask, out_val;  // controls outside the tile (state bits)
};

// A run of gates applied between two barriers: kind 0 = a register group on
// the R tile positions p[] (ascending), kind 1 = one gate through the
// per-gate shared-memory paths.
struct FGroup {
    uint8_t kind;
    uint8_t p[4];
    uint8_t pad[3];
    uint16_t first, count;
};

// Split a launch's gates into register groups (1-target gates whose targets
// and in-tile controls span at most R tile positions, padded with the lowest
// unused positions) and single gates, and fill the local target and control
// fields of grouped gates.  Gates on disjoint tile positions commute, so a
// group may take any later gate whose earlier conflicting gates are all
// placed: starting from the first unplaced gate, a group first takes every
// such gate inside its position set, then grows the set by the gate adding
// the fewest positions, up to R.  (A layer of 1-qubit gates followed by a CNOT
// chain becomes two groups instead of one per run of consecutive gates.)
// The gates and their integer-pipe constants are permuted into group order;
// returns the number of groups.
template <class KC>
inline int group_fused_gates(FGate *gates, KC *kc, int cnt, int k, int R, FGroup *groups) {
    std::vector<uint32_t> P(size_t(cnt) + 1);
    for (int i = 0; i < cnt; i++) {
        const FGate &g = gates[i];
        P[size_t(i)] = g.in_mask | (1u << g.q0) | (g.ntgt == 2 ? (1u << g.q1) : 0u);
    }
    auto groupable = [&](int i) { return k >= R && gates[i].ntgt == 1 && __builtin_popcount(P[size_t(i)]) <= R; };
    std::vector<char> done(size_t(cnt) + 1, 0);
    auto ready = [&](int i) {
        for (int h = 0; h < i; h++)
            if (!done[size_t(h)] && (P[size_t(h)] & P[size_t(i)])) return false;
        return true;
    };
    std::vector<int> order;
    order.reserve(size_t(cnt));
    int ng = 0;
    int first = 0;
    while (true) {
        while (first < cnt && done[size_t(first)]) first++;
        if (first >= cnt) break;
        const int i0 = first;  // every earlier gate is placed
        const uint16_t start = uint16_t(order.size());
        done[size_t(i0)] = 1;
        order.push_back(i0);
        if (!groupable(i0)) {
            groups[ng++] = FGroup{1, {0, 0, 0, 0}, {0, 0, 0}, start, 1};
            continue;
        }
        uint32_t set = P[size_t(i0)];
        for (;;) {
            bool added = false;
            for (int i = i0 + 1; i < cnt; i++)
                if (!done[size_t(i)] && groupable(i) && (P[size_t(i)] & ~set) == 0 && ready(i)) {
                    done[size_t(i)] = 1;
                    order.push_back(i);
                    added = true;
                }
            if (added) continue;
            int best = -1, best_n = R + 1;
            for (int i = i0 + 1; i < cnt; i++)
                if (!done[size_t(i)] && groupable(i) && ready(i)) {
                    const int c = __builtin_popcount(set | P[size_t(i)]);
                    if (c < best_n) {
                        best = i;
                        best_n = c;
                    }
                }
            if (best < 0 || best_n > R) break;
            set |= P[size_t(best)];
            done[size_t(best)] = 1;
            order.push_back(best);
        }
        const int count = int(order.size()) - int(start);
        if (count == 1) {  // a lone gate touches only its own pairs through the per-gate path
            groups[ng++] = FGroup{1, {0, 0, 0, 0}, {0, 0, 0}, start, 1};
            continue;
        }
        for (int q = 0; q < k && __builtin_popcount(set) < R; q++) set |= 1u << q;
        FGroup G{0, {0, 0, 0, 0}, {0, 0, 0}, start, uint16_t(count)};
        int nb = 0;
        for (int q = 0; q < k; q++)
            if ((set >> q) & 1u) G.p[nb++] = uint8_t(q);
        groups[ng++] = G;
    }
    // permute into group order, then fill the local fields of grouped gates
    std::vector<FGate> g2(gates, gates + cnt);
    std::vector<unsigned char> k2(sizeof(KC) * size_t(cnt));
    std::memcpy(k2.data(), kc, k2.size());
    for (int i = 0; i < cnt; i++) {
        gates[i] = g2[size_t(order[size_t(i)])];
        std::memcpy(&kc[i], k2.data() + sizeof(KC) * size_t(order[size_t(i)]), sizeof(KC));
    }
    for (int gr = 0; gr < ng; gr++) {
        const FGroup &G = groups[gr];
        if (G.kind != 0) continue;
        int loc[32];
        for (int b = 0; b < R; b++) loc[G.p[b]] = b;
        for (int t = G.first; t < G.first + G.count; t++) {
            FGate &g = gates[t];
            g.lt = uint8_t(loc[g.q0]);
            g.lcm = 0;
            g.lcv = 0;
            for (int q = 0; q < k; q++)
                if ((g.in_mask >> q) & 1u) {
                    g.lcm |= uint8_t(1u << loc[q]);
                    if ((g.in_val >> q) & 1u) g.lcv |= uint8_t(1u << loc[q]);
                }
        }
    }
    return ng;
}

// A dense unitary 1-target gate U (all four entries non-zero, some entry not
// real, not of the RX form [[a, -ib], [-ib, a]]) as D_L R D_R, applied D_R
// first: R = [[c, -s], [s, c]] real, D_R = diag(1, e^{i r}), D_L =
// diag(e^{i l0}, e^{i l1}) with c = |U00|, s = |U10|, l0 = arg U00, l1 =
// arg U10, r = arg(-U01) - l0.  The product matches U00, U01 and U10 by
// construction and U11 through unitarity (U11 = det U conj(U00)); the split
// is taken only when the product reproduces U within 1e-13.  Controls carry
// over (a controlled product is the product of the controlled factors).  R
// takes the real body, about half the float-float operations of the dense
// body, and the diagonals can fold into phase tables.
inline bool split_dense_1q(const lgpu_fused_gate_t &g, lgpu_fused_gate_t f[3]) {
    using cd = std::complex<double>;
    if (g.ntgt != 1) return false;
    const cd a(g.m[0], g.m[1]), b(g.m[2], g.m[3]), c(g.m[4], g.m[5]), d(g.m[6], g.m[7]);
    if (a == 0.0 || b == 0.0 || c == 0.0 || d == 0.0) return false;
    if (a.imag() == 0 && b.imag() == 0 && c.imag() == 0 && d.imag() == 0) return false;  // real body already
    if (a.imag() == 0 && d.imag() == 0 && a.real() == d.real() && b.real() == 0 && c.real() == 0) return false;
    const double cc = std::abs(a), ss = std::abs(c);
    const double l0 = std::arg(a), l1 = std::arg(c), r = std::arg(-b) - l0;
    const cd eL0 = std::polar(1.0, l0), eL1 = std::polar(1.0, l1), eR = std::polar(1.0, r);
    const cd q[4] = {eL0 * cc, -eL0 * ss * eR, eL1 * ss, eL1 * cc * eR};
    const cd u[4] = {a, b, c, d};
    for (int e = 0; e < 4; e++)
        if (std::abs(q[e] - u[e]) > 1e-13) return false;
    for (int k = 0; k < 3; k++) {
        f[k] = g;
        for (double &x : f[k].m) x = 0.0;
    }
    f[0].m[0] = 1.0;
    f[0].m[6] = eR.real();
    f[0].m[7] = eR.imag();
    f[1].m[0] = cc;
    f[1].m[2] = -ss;
    f[1].m[4] = ss;
    f[1].m[6] = cc;
    f[2].m[0] = eL0.real();
    f[2].m[1] = eL0.imag();
    f[2].m[6] = eL1.real();
    f[2].m[7] = eL1.imag();
    return true;
}

// Diagonal gates of a float-float block folded into phase tables.  A 1-target
// gate whose 2x2 is diagonal (other than diag(+-1, +-1), which stays a sign
// flip), with its controls (if any) on tile bits, is a diagonal on its
// support (target and controls).  It commutes with every diagonal gate and
// with every gate that targets none of its support bits (controls are
// diagonal), so it may run at any point between the nearest such blocking
// gates before and after it.  Folding places groups of these gates at common
// points (interval stabbing: the unplaced gate whose interval ends first
// fixes the point, at that end, and every unplaced gate whose interval holds
// the point joins while the union of the supports stays within
// kDiagTableBits); a group is one table of 2^k phases over the union of its
// supports.  A group of one gate stays that gate, in place.
//
// With split_dense, dense 1-target unitaries are first split by
// split_dense_1q so that their diagonals can join the tables.  A split is
// kept only while its estimated cost (a real body plus its diagonals, each a
// table share or a diagonal body of its own) stays below the dense body's,
// and only if the splits add no launch (kFusedMaxGates records per launch).
// Cost units are float-float instructions per amplitude pair, shared-memory
// pass included: dense body 110, real body 54, diagonal body 56, table 66.
//
// A folded group is returned as a record with ntgt = kDiagTableMark, its
// support bits in ctrl[0..k-1] in ascending tile position (table index bit b
// = ctrl[b]) and the table in m (entry i = m[2i] + i m[2i+1]); internal[i]
// marks those records.
inline std::vector<lgpu_fused_gate_t> fold_diagonal_gates(const lgpu_fused_gate_t *gates, uint32_t ngates,
                                                          const std::vector<int> &pos, std::vector<char> &internal,
                                                          bool split_dense = false) {
    using cd = std::complex<double>;
    const int n = int(pos.size());
    auto foldable = [&](const lgpu_fused_gate_t &g, uint64_t *support) {
        if (g.ntgt != 1 || g.nctrl < 0 || g.nctrl > kDiagTableBits - 1) return false;
        for (int e = 2; e < 6; e++)
            if (g.m[e] != 0.0) return false;  // off-diagonal entries
        // diag(+-1, +-1) (Z, CZ) stays a sign flip, cheaper than a table entry
        auto pm1 = [](double v) { return v == 1.0 || v == -1.0; };
        if (pm1(g.m[0]) && g.m[1] == 0.0 && pm1(g.m[6]) && g.m[7] == 0.0) return false;
        uint64_t sb = 0;
        auto add = [&](int b) {
            if (b < 0 || b >= n || pos[size_t(b)] < 0 || ((sb >> b) & 1u)) return false;
            sb |= uint64_t(1) << b;
            return true;
        };
        if (!add(g.tgt[0])) return false;
        for (int c = 0; c < g.nctrl; c++)
            if (!add(g.ctrl[c])) return false;
        *support = sb;
        return true;
    };
    // bits a gate acts on non-diagonally (all bits when unknown); 0 for a diagonal 2x2
    auto blocks = [](const lgpu_fused_gate_t &g) -> uint64_t {
        if (g.ntgt == 1 && g.m[2] == 0.0 && g.m[3] == 0.0 && g.m[4] == 0.0 && g.m[5] == 0.0) return 0;
        if (g.ntgt < 1 || g.ntgt > 2) return ~uint64_t(0);
        uint64_t t = 0;
        for (int j = 0; j < g.ntgt; j++) {
            if (g.tgt[j] < 0 || g.tgt[j] >= 64) return ~uint64_t(0);
            t |= uint64_t(1) << g.tgt[j];
        }
        return t;
    };
    struct Item {
        lgpu_fused_gate_t g;
        int origin;  // index of the split source gate (-1: an input gate)
        int part;    // 0 = D_R, 1 = R, 2 = D_L of a split
    };
    struct Fold {
        std::vector<Item> list;
        std::vector<int> group;     // per item: its group, or -1
        std::vector<int> slot;      // per group: placed before item slot (list size: at the end)
        std::vector<uint64_t> sup;  // per group: support bits
        std::vector<std::vector<int>> members;
        size_t records = 0;
    };
    auto run = [&](const std::vector<char> &split) {
        Fold F;
        for (uint32_t i = 0; i < ngates; i++) {
            lgpu_fused_gate_t parts[3];
            if (split[i] && split_dense_1q(gates[i], parts)) {
                for (int k = 0; k < 3; k++) F.list.push_back(Item{parts[k], int(i), k});
            } else {
                F.list.push_back(Item{gates[i], -1, 0});
            }
        }
        const int N = int(F.list.size());
        std::vector<uint64_t> S(size_t(N), 0), B(size_t(N), 0);
        std::vector<char> fold(size_t(N), 0);
        for (int i = 0; i < N; i++) {
            fold[size_t(i)] = foldable(F.list[size_t(i)].g, &S[size_t(i)]) ? 1 : 0;
            B[size_t(i)] = blocks(F.list[size_t(i)].g);
        }
        std::vector<int> lo(size_t(N), 0), hi(size_t(N), N), cand;
        for (int i = 0; i < N; i++) {
            if (!fold[size_t(i)]) continue;
            for (int j = i - 1; j >= 0; j--)
                if (B[size_t(j)] & S[size_t(i)]) {
                    lo[size_t(i)] = j + 1;
                    break;
                }
            for (int j = i + 1; j < N; j++)
                if (B[size_t(j)] & S[size_t(i)]) {
                    hi[size_t(i)] = j;
                    break;
                }
            cand.push_back(i);
        }
        std::stable_sort(cand.begin(), cand.end(), [&](int a, int b) { return hi[size_t(a)] < hi[size_t(b)]; });
        F.group.assign(size_t(N), -1);
        for (size_t ci = 0; ci < cand.size(); ci++) {
            const int d = cand[ci];
            if (F.group[size_t(d)] >= 0) continue;
            const int gid = int(F.slot.size());
            const int p = hi[size_t(d)];
            uint64_t sup = S[size_t(d)];
            std::vector<int> mem{d};
            F.group[size_t(d)] = gid;
            for (size_t cj = ci + 1; cj < cand.size(); cj++) {
                const int e = cand[cj];
                if (F.group[size_t(e)] >= 0 || lo[size_t(e)] > p) continue;
                if (__builtin_popcountll(sup | S[size_t(e)]) > kDiagTableBits) continue;
                sup |= S[size_t(e)];
                mem.push_back(e);
                F.group[size_t(e)] = gid;
            }
            F.slot.push_back(p);
            F.sup.push_back(sup);
            F.members.push_back(mem);
        }
        size_t tables = 0;
        for (const auto &m : F.members) tables += m.size() >= 2;
        size_t folded_away = 0;
        for (const auto &m : F.members)
            if (m.size() >= 2) folded_away += m.size();
        F.records = size_t(N) - folded_away + tables;
        return F;
    };
    // estimated cost of a split (see above) against the dense body's 110
    auto split_cost = [&](const Fold &F, int origin) {
        double c = 54.0;
        for (size_t i = 0; i < F.list.size(); i++) {
            if (F.list[i].origin != origin || F.list[i].part == 1) continue;
            const int gid = F.group[i];
            const size_t k = gid >= 0 ? F.members[size_t(gid)].size() : 1;
            c += k >= 2 ? 66.0 / double(k) : 56.0;
        }
        return c;
    };
    std::vector<char> split(ngates, 0);
    Fold F = run(split);
    if (split_dense) {
        bool any = false;
        for (uint32_t i = 0; i < ngates; i++) {
            lgpu_fused_gate_t parts[3];
            split[i] = split_dense_1q(gates[i], parts) ? 1 : 0;
            any = any || split[i];
        }
        if (any) {
            const size_t launches0 = (F.records + kFusedMaxGates - 1) / kFusedMaxGates;
            Fold S = run(split);
            for (int it = 0; it < 64; it++) {  // drop the splits that do not pay, then refold
                bool changed = false;
                for (uint32_t i = 0; i < ngates; i++)
                    if (split[i] && split_cost(S, int(i)) >= 110.0) {
                        split[i] = 0;
                        changed = true;
                    }
                if (!changed) break;
                S = run(split);
            }
            bool kept = false;
            for (uint32_t i = 0; i < ngates; i++) kept = kept || split[i];
            if (kept && (S.records + kFusedMaxGates - 1) / kFusedMaxGates <= launches0) F = std::move(S);
        }
    }
    // emit: the tables placed before item p, then item p unless it was folded
    const int N = int(F.list.size());
    std::vector<lgpu_fused_gate_t> out;
    internal.clear();
    auto emit_table = [&](size_t gid) {
        std::vector<int> bits;  // support bits in ascending tile position
        for (int b = 0; b < n; b++)
            if ((F.sup[gid] >> b) & 1u) bits.push_back(b);
        std::sort(bits.begin(), bits.end(), [&](int a, int b) { return pos[size_t(a)] < pos[size_t(b)]; });
        const int k = int(bits.size());
        lgpu_fused_gate_t r{};
        r.ntgt = kDiagTableMark;
        r.nctrl = k;
        for (int b = 0; b < k; b++) r.ctrl[b] = bits[size_t(b)];
        for (int idx = 0; idx < (1 << kDiagTableBits); idx++) {
            cd t = idx < (1 << k) ? cd(1.0, 0.0) : cd(0.0, 0.0);
            if (idx < (1 << k)) {
                auto bit = [&](int state_bit) {
                    for (int b = 0; b < k; b++)
                        if (bits[size_t(b)] == state_bit) return (idx >> b) & 1;
                    return 0;
                };
                for (int mi : F.members[gid]) {
                    const lgpu_fused_gate_t &g = F.list[size_t(mi)].g;
                    bool on = true;
                    for (int c = 0; c < g.nctrl; c++)
                        if (bit(g.ctrl[c]) != (g.ctrl_val[c] ? 1 : 0)) on = false;
                    if (!on) continue;
                    t *= bit(g.tgt[0]) ? cd(g.m[6], g.m[7]) : cd(g.m[0], g.m[1]);
                }
            }
            r.m[2 * idx] = t.real();
            r.m[2 * idx + 1] = t.imag();
        }
        out.push_back(r);
        internal.push_back(1);
    };
    std::vector<std::vector<size_t>> at(size_t(N) + 1);
    for (size_t gid = 0; gid < F.members.size(); gid++)
        if (F.members[gid].size() >= 2) at[size_t(F.slot[gid])].push_back(gid);
    for (int p = 0; p <= N; p++) {
        for (size_t gid : at[size_t(p)]) emit_table(gid);
        if (p == N) break;
        const int gid = F.group[size_t(p)];
        if (gid >= 0 && F.members[size_t(gid)].size() >= 2) continue;
        out.push_back(F.list[size_t(p)].g);
        internal.push_back(0);
    }
    return out;
}

}  // namespace lgpu
