// Host-side plan of the Pauli-word tile passes: which words share one read
// of the state.  Plain C++ (no CUDA types), so it can be unit-tested on the
// host.
#pragma once

#include <algorithm>
#include <cstdint>
#include <vector>

namespace lgpu {

constexpr int kTileWords = 8;  // words per pass: their per-thread accumulators stay in registers
constexpr int kTileHiMax = 8;  // tile bits above the low run (runs of a tile: at most 2^8)

// A tile is the low run of state bits 0..m-1 (m >= mmin, so that each run of
// 2^m amplitudes the tile gathers is long enough for full memory
// transactions) plus at most kTileHiMax higher bits, kmax bits in all (kmax
// when n >= kmax: the largest m that leaves room for the high bits is taken).
// A pass holds up to kTileWords words whose flip bits all lie in its tile.
// Words are placed first-fit in decreasing order of their flip-bit count (the
// widest first; diagonal words fill the slots left over), each pass lists its
// words in ascending order, and words whose flips fit no tile are left out.
struct TilePass {
    std::vector<int> tile;
    std::vector<uint32_t> words;
};

// The tile for a flip-bit union, or false when none holds it.
inline bool tile_for_mask(uint32_t n, uint64_t mask, int kmax, int mmin, std::vector<int> &tile) {
    for (int m = std::min<int>(kmax, int(n)); m >= std::min<int>(mmin, kmax); m--) {
        std::vector<int> hi;
        for (int b = m; b < int(n); b++)
            if ((mask >> b) & 1u) hi.push_back(b);
        if (int(hi.size()) <= kmax - m && int(hi.size()) <= kTileHiMax) {
            tile.clear();
            for (int b = 0; b < m; b++) tile.push_back(b);
            tile.insert(tile.end(), hi.begin(), hi.end());
            return true;
        }
    }
    return false;
}

inline std::vector<TilePass> plan_tile_passes(uint32_t n, uint32_t nwords, const uint64_t *flip, int kmax, int mmin) {
    std::vector<uint32_t> order(nwords);
    for (uint32_t w = 0; w < nwords; w++) order[w] = w;
    std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) {
        return __builtin_popcountll(flip[a]) > __builtin_popcountll(flip[b]);
    });
    std::vector<TilePass> passes;
    std::vector<uint64_t> unions;
    std::vector<int> t;
    for (uint32_t w : order) {
        bool placed = false;
        for (size_t pi = 0; pi < passes.size() && !placed; pi++) {
            if (passes[pi].words.size() >= size_t(kTileWords)) continue;
            if (tile_for_mask(n, unions[pi] | flip[w], kmax, mmin, t)) {
                unions[pi] |= flip[w];
                passes[pi].tile = t;
                passes[pi].words.push_back(w);
                placed = true;
            }
        }
        if (!placed) {
            TilePass tp;
            if (!tile_for_mask(n, flip[w], kmax, mmin, tp.tile)) continue;  // flips too many bits: left to the caller
            tp.words.push_back(w);
            passes.push_back(tp);
            unions.push_back(flip[w]);
        }
    }
    for (auto &p : passes) std::sort(p.words.begin(), p.words.end());
    return passes;
}

}  // namespace lgpu
