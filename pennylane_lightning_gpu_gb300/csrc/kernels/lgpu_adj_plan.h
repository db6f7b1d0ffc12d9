// Phase groups of the adjoint blocks: which steps of a run are
// gathered into one group step, and in what order the steps then run.  Plain
// C++ (no CUDA types), so the plan can be checked on the host.
#pragma once

#include <cstdint>
#include <vector>

namespace lgpu {

// What the plan needs to know of a step.
struct AdjPlanStep {
    int q;           // tile position of the target
    bool groupable;  // uncontrolled, diagonal U^dag, generator none, Z or P1
    bool diagonal;   // U^dag diagonal (controls allowed)
    bool grad;       // has a gradient
};

// Groups of uncontrolled diagonal steps on at most max_bits tile positions,
// at most max_grads of them with a gradient.  A group starts at such a step
// and takes later ones moved back past the steps in between: a diagonal step
// commutes (with its generator, Z or P1) with every diagonal step and with
// every step that targets another position (controls are diagonal), so only
// a non-diagonal step on its position blocks the move.  The steps left behind
// keep their order.  Returns the new order: one entry per step or group (the
// steps of a group in their original order); a group has two or more steps.
inline std::vector<std::vector<uint32_t>> plan_phase_groups(const std::vector<AdjPlanStep> &in, int max_bits,
                                                           int max_grads) {
    const uint32_t n = uint32_t(in.size());
    std::vector<std::vector<uint32_t>> out;
    std::vector<char> used(n, 0);
    for (uint32_t i = 0; i < n; i++) {
        if (used[i]) continue;
        if (!in[i].groupable) {
            out.push_back({i});
            continue;
        }
        std::vector<uint32_t> mem{i};
        uint64_t pm = uint64_t(1) << in[i].q, blocked = 0;
        int ng = in[i].grad ? 1 : 0;
        for (uint32_t j = i + 1; j < n; j++) {
            if (used[j]) continue;
            const AdjPlanStep &st = in[j];
            const uint64_t bit = uint64_t(1) << st.q;
            const bool can = st.groupable && !(blocked & bit) && __builtin_popcountll(pm | bit) <= max_bits &&
                             ng + (st.grad ? 1 : 0) <= max_grads;
            if (can) {
                mem.push_back(j);
                pm |= bit;
                ng += st.grad ? 1 : 0;
            } else if (!st.diagonal) {
                blocked |= bit;  // later steps on this position stay behind it
            }
        }
        if (mem.size() < 2) {
            out.push_back({i});
            continue;
        }
        for (uint32_t r : mem) used[r] = 1;
        out.push_back(mem);
    }
    return out;
}

}  // namespace lgpu
