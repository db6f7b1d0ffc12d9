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

// Diagonal gates of a float-float block folded into phase tables.  A 1-target
// gate whose 2x2 is diagonal (other than diag(+-1, +-1), which stays a sign
// flip), with its controls (if any) on tile bits, is a diagonal on its
// support (target and controls).  Such gates join a group
// whose product is one table of 2^k phases over the union of the supports
// (k <= kDiagTableBits), applied where the group's first gate stood.  A later
// gate may join only if no gate between them targets a bit of its support
// (diagonal gates commute with each other and with controls), so moving it
// back changes nothing.  A group of one gate stays that gate.  A folded group
// is returned as a record with ntgt = kDiagTableMark, its support bits in
// ctrl[0..k-1] in ascending tile position (table index bit b = ctrl[b]) and the
// table in m (entry i = m[2i] + i m[2i+1]); internal[i] marks those records.
inline std::vector<lgpu_fused_gate_t> fold_diagonal_gates(const lgpu_fused_gate_t *gates, uint32_t ngates,
                                                          const std::vector<int> &pos, std::vector<char> &internal) {
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
    struct Group {
        size_t slot;  // index in out
        uint64_t support;
        std::vector<uint32_t> members;
    };
    std::vector<lgpu_fused_gate_t> out;
    std::vector<Group> groups;
    internal.clear();
    int open = -1;         // the group later diagonal gates may join
    uint64_t blocked = 0;  // bits targeted by other gates since the open group's first gate
    for (uint32_t i = 0; i < ngates; i++) {
        const lgpu_fused_gate_t &g = gates[i];
        uint64_t sb = 0;
        if (foldable(g, &sb)) {
            if (open >= 0 && (sb & blocked) == 0 &&
                __builtin_popcountll(groups[size_t(open)].support | sb) <= kDiagTableBits) {
                groups[size_t(open)].support |= sb;
                groups[size_t(open)].members.push_back(i);
                continue;
            }
            open = int(groups.size());
            groups.push_back(Group{out.size(), sb, {i}});
            out.push_back(g);  // replaced below if the group takes more gates
            internal.push_back(0);
            blocked = 0;
            continue;
        }
        out.push_back(g);
        internal.push_back(0);
        // a gate whose matrix is not diagonal blocks its targets
        const bool diag1 = g.ntgt == 1 && g.m[2] == 0.0 && g.m[3] == 0.0 && g.m[4] == 0.0 && g.m[5] == 0.0;
        if (!diag1)
            for (int t = 0; t < g.ntgt && t < 2; t++)
                if (g.tgt[t] >= 0 && g.tgt[t] < 64) blocked |= uint64_t(1) << g.tgt[t];
    }
    for (const Group &G : groups) {
        if (G.members.size() < 2) continue;
        std::vector<int> bits;  // support bits in ascending tile position
        for (int b = 0; b < n; b++)
            if ((G.support >> b) & 1u) bits.push_back(b);
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
                for (uint32_t mi : G.members) {
                    const lgpu_fused_gate_t &g = gates[mi];
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
        out[G.slot] = r;
        internal[G.slot] = 1;
    }
    return out;
}

}  // namespace lgpu
