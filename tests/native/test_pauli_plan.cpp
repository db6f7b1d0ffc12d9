// Host test of the Pauli-word tile pass plan (lgpu_pauli_plan.h): random
// flip masks of 1..9 bits on 16..30-qubit states, tiles of 11 and 12 bits.
// Checks: every word whose flip mask fits a tile on its own lands in exactly
// one pass, the others in none; a pass holds 1..kTileWords words in
// ascending order; its tile is the low run 0..m-1 (m >= 5) plus at most 6
// higher bits, at most kmax bits in all, and holds the flip bits of all its
// words.
#include <algorithm>
#include <cstdio>
#include <random>
#include <vector>

#include "lgpu_pauli_plan.h"

static long bad = 0;

static void fail(const char *what, int trial, long v) {
    if (bad < 20) std::printf("bad %s (trial %d): %ld\n", what, trial, v);
    bad++;
}

// Whether a flip mask fits a tile on its own (the planner's rule).
static bool fits(uint64_t mask, int n, int kmax) {
    for (int m = std::min(kmax, n); m >= std::min(5, kmax); m--) {
        int hi = 0;
        for (int b = m; b < n; b++)
            if ((mask >> b) & 1u) hi++;
        if (hi <= kmax - m && hi <= 6) return true;
    }
    return false;
}

int main() {
    std::mt19937_64 gen(5);
    long nwords_total = 0, npasses = 0, nleft = 0;
    int trial = 0;
    for (int n = 16; n <= 30; n += 2) {
        for (int kmax : {11, 12}) {
            for (int rep = 0; rep < 60; rep++, trial++) {
                const uint32_t nw = 1 + uint32_t(gen() % 120);
                std::vector<uint64_t> flip(nw);
                for (auto &f : flip) {
                    f = 0;
                    const int nb = int(gen() % 10);  // 0: a diagonal word
                    for (int k = 0; k < nb; k++) f |= uint64_t(1) << (gen() % uint64_t(n));
                }
                const auto passes = lgpu::plan_tile_passes(uint32_t(n), nw, flip.data(), kmax);
                std::vector<int> seen(nw, 0);
                for (const auto &p : passes) {
                    npasses++;
                    if (p.words.empty() || p.words.size() > size_t(lgpu::kTileWords))
                        fail("pass size", trial, long(p.words.size()));
                    int m = 0;
                    while (m < int(p.tile.size()) && p.tile[size_t(m)] == m) m++;
                    if (m < 5) fail("low run shorter than 5", trial, m);
                    if (p.tile.size() - size_t(m) > 6) fail("more than 6 high bits", trial, long(p.tile.size()));
                    if (int(p.tile.size()) > kmax) fail("tile larger than kmax", trial, long(p.tile.size()));
                    uint64_t tmask = 0;
                    for (int b : p.tile) tmask |= uint64_t(1) << b;
                    for (size_t i = 0; i < p.words.size(); i++) {
                        const uint32_t w = p.words[i];
                        if (w >= nw) {
                            fail("word index", trial, long(w));
                            continue;
                        }
                        if (i > 0 && w <= p.words[i - 1]) fail("words not ascending", trial, long(w));
                        seen[w]++;
                        if (flip[w] & ~tmask) fail("flip bit outside the tile", trial, long(w));
                    }
                }
                for (uint32_t w = 0; w < nw; w++) {
                    const bool f = fits(flip[w], n, kmax);
                    if (f && seen[w] != 1) fail("fitting word not planned exactly once", trial, long(w));
                    if (!f && seen[w] != 0) fail("word planned although it fits no tile", trial, long(w));
                    if (!f) nleft++;
                }
                nwords_total += nw;
            }
        }
    }
    std::printf("plans %d words %ld passes %ld left to the flip-mask passes %ld bad %ld\n", trial, nwords_total,
                npasses, nleft, bad);
    return bad == 0 ? 0 : 1;
}
