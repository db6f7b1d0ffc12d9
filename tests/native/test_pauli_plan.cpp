// Host test of the Pauli-word tile pass plan (lgpu_pauli_plan.h): random
// flip masks of 1..9 bits on 16..30-qubit states, tiles of 11 and 12 bits.
// Checks: every word whose flip mask fits a tile on its own lands in exactly
// one pass, the others in none; a pass holds 1..kTileWords words in
// ascending order; its tile is the low run 0..m-1 (m >= mmin) plus at most
// kTileHiMax higher bits, exactly kmax bits in all (n >= kmax), and holds the
// flip bits of all its words.  Also: the first-fit-decreasing order packs the
// words of a 100-word random Hamiltonian on 28 qubits into no more passes
// than first-fit in word order.
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
static bool fits(uint64_t mask, int n, int kmax, int mmin) {
    for (int m = std::min(kmax, n); m >= std::min(mmin, kmax); m--) {
        int hi = 0;
        for (int b = m; b < n; b++)
            if ((mask >> b) & 1u) hi++;
        if (hi <= kmax - m && hi <= lgpu::kTileHiMax) return true;
    }
    return false;
}

// First-fit in word order (no sorting), for the pass-count comparison.
static size_t first_fit_passes(uint32_t n, const std::vector<uint64_t> &flip, int kmax, int mmin) {
    std::vector<uint64_t> unions;
    std::vector<size_t> sizes;
    std::vector<int> t;
    for (uint64_t f : flip) {
        bool placed = false;
        for (size_t i = 0; i < unions.size() && !placed; i++)
            if (sizes[i] < size_t(lgpu::kTileWords) && lgpu::tile_for_mask(n, unions[i] | f, kmax, mmin, t)) {
                unions[i] |= f;
                sizes[i]++;
                placed = true;
            }
        if (!placed && lgpu::tile_for_mask(n, f, kmax, mmin, t)) {
            unions.push_back(f);
            sizes.push_back(1);
        }
    }
    return unions.size();
}

int main() {
    std::mt19937_64 gen(5);
    long nwords_total = 0, npasses = 0, nleft = 0;
    int trial = 0;
    for (int n = 16; n <= 30; n += 2) {
        for (int kmax : {11, 12}) {
            const int mmin = kmax == 11 ? 3 : 4;
            for (int rep = 0; rep < 60; rep++, trial++) {
                const uint32_t nw = 1 + uint32_t(gen() % 120);
                std::vector<uint64_t> flip(nw);
                for (auto &f : flip) {
                    f = 0;
                    const int nb = int(gen() % 10);  // 0: a diagonal word
                    for (int k = 0; k < nb; k++) f |= uint64_t(1) << (gen() % uint64_t(n));
                }
                const auto passes = lgpu::plan_tile_passes(uint32_t(n), nw, flip.data(), kmax, mmin);
                std::vector<int> seen(nw, 0);
                for (const auto &p : passes) {
                    npasses++;
                    if (p.words.empty() || p.words.size() > size_t(lgpu::kTileWords))
                        fail("pass size", trial, long(p.words.size()));
                    int m = 0;
                    while (m < int(p.tile.size()) && p.tile[size_t(m)] == m) m++;
                    if (m < mmin) fail("low run shorter than mmin", trial, m);
                    if (p.tile.size() - size_t(m) > size_t(lgpu::kTileHiMax))
                        fail("too many high bits", trial, long(p.tile.size()));
                    if (int(p.tile.size()) != kmax) fail("tile not of kmax bits", trial, long(p.tile.size()));
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
                    const bool f = fits(flip[w], n, kmax, mmin);
                    if (f && seen[w] != 1) fail("fitting word not planned exactly once", trial, long(w));
                    if (!f && seen[w] != 0) fail("word planned although it fits no tile", trial, long(w));
                    if (!f) nleft++;
                }
                nwords_total += nw;
            }
        }
    }
    // 100 words of 1..6 distinct wires, each X, Y or Z, on 28 qubits
    long ffd = 0, ff = 0;
    for (int rep = 0; rep < 40; rep++) {
        std::vector<uint64_t> flip(100);
        for (auto &f : flip) {
            f = 0;
            const int nb = 1 + int(gen() % 6);
            uint64_t used = 0;
            for (int k = 0; k < nb; k++) {
                int b;
                do b = int(gen() % 28);
                while ((used >> b) & 1u);
                used |= uint64_t(1) << b;
                if (gen() % 3 != 2) f |= uint64_t(1) << b;  // X or Y flips, Z does not
            }
        }
        const size_t a = lgpu::plan_tile_passes(28, 100, flip.data(), 11, 3).size();
        const size_t b = first_fit_passes(28, flip, 11, 3);
        ffd += long(a);
        ff += long(b);
    }
    if (ffd > ff) fail("decreasing order needs more passes than word order", 0, ffd - ff);
    std::printf("plans %d words %ld passes %ld left to the flip-mask passes %ld; 100-word sets: %ld passes "
                "(word order %ld) bad %ld\n",
                trial, nwords_total, npasses, nleft, ffd, ff, bad);
    return bad == 0 ? 0 : 1;
}
