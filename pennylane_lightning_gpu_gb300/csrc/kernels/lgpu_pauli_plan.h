// Host-side plan of the Pauli-word tile passes: which words share one read
// of the state.  Plain C++ (no CUDA types), so it can be unit-tested on the
// host.
#pragma once

#include <algorithm>
#include <cstdint>
#include <vector>

namespace lgpu {

constexpr int kTileWords = 8;  // words per pass: their per-thread accumulators stay in registers

// Group words into tile passes: a word joins the first pass whose tile can
// also hold its flip bits (low run >= 5 bits, <= 6 high bits, <= kmax bits).
struct TilePass {
    std::vector<int> tile;
    std::vector<uint32_t> words;
};
inline std::vector<TilePass> plan_tile_passes(uint32_t n, uint32_t nwords, const uint64_t *flip, int kmax) {
    std::vector<TilePass> passes;
    std::vector<uint64_t> unions;
    auto tile_of = [&](uint64_t mask, std::vector<int> &tile) {
        for (int m = std::min<int>(kmax, int(n)); m >= std::min<int>(5, kmax); m--) {
            std::vector<int> hi;
            for (int b = m; b < int(n); b++)
                if ((mask >> b) & 1u) hi.push_back(b);
            if (int(hi.size()) <= kmax - m && hi.size() <= 6) {
                tile.clear();
                for (int b = 0; b < m; b++) tile.push_back(b);
                tile.insert(tile.end(), hi.begin(), hi.end());
                return true;
            }
        }
        return false;
    };
    for (uint32_t w = 0; w < nwords; w++) {
        bool placed = false;
        for (size_t pi = 0; pi < passes.size() && !placed; pi++) {
            if (passes[pi].words.size() >= size_t(kTileWords)) continue;
            std::vector<int> t;
            if (tile_of(unions[pi] | flip[w], t)) {
                unions[pi] |= flip[w];
                passes[pi].tile = t;
                passes[pi].words.push_back(w);
                placed = true;
            }
        }
        if (!placed) {
            TilePass tp;
            if (!tile_of(flip[w], tp.tile)) continue;  // flips too many bits: left to the caller
            tp.words.push_back(w);
            passes.push_back(tp);
            unions.push_back(flip[w]);
        }
    }
    return passes;
}

}  // namespace lgpu
