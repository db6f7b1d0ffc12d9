// Host test of the folding of diagonal gates into phase tables
// (lgpu_fused_plan.h::fold_diagonal_gates), which the float-float fused blocks
// apply instead of the gates, without and with the split of dense 1-target
// unitaries (split_dense_1q): on random blocks (1-target gates, diagonal,
// dense unitary or general, with controls inside or outside the tile, and
// 2-target gates) the folded list must transform random states as the
// original list does (within 1e-12), every table must cover at most
// kDiagTableBits tile positions, the records must be flagged as folded
// exactly when they are tables, diag(+-1, +-1) gates must stay as they are,
// and the splits must add no launch of kFusedMaxGates records.  Layer-shaped
// blocks (dense unitaries on every tile bit, then CNOTs) must keep splits.
// split_dense_1q's edge cases are checked on their own (split_edge_cases).
#include <cmath>
#include <complex>
#include <cstdio>
#include <random>
#include <vector>

#include "lgpu_fused_plan.h"

using cd = std::complex<double>;
static long bad = 0;

static void fail(const char *what, int trial, double v) {
    if (bad < 20) std::printf("bad %s (trial %d): %g\n", what, trial, v);
    bad++;
}

static bool controls_on(const lgpu_fused_gate_t &g, uint64_t i) {
    for (int c = 0; c < g.nctrl; c++)
        if (((i >> g.ctrl[c]) & 1u) != uint64_t(g.ctrl_val[c] ? 1 : 0)) return false;
    return true;
}

static void apply(std::vector<cd> &v, const lgpu_fused_gate_t &g, bool table) {
    const uint64_t N = v.size();
    auto m = [&](int r, int c, int d) { return cd(g.m[2 * (r * d + c)], g.m[2 * (r * d + c) + 1]); };
    if (table) {  // phase table over ctrl[0..nctrl-1], index bit b = ctrl[b]
        for (uint64_t i = 0; i < N; i++) {
            int idx = 0;
            for (int b = 0; b < g.nctrl; b++) idx |= int((i >> g.ctrl[b]) & 1u) << b;
            v[i] *= cd(g.m[2 * idx], g.m[2 * idx + 1]);
        }
        return;
    }
    if (g.ntgt == 1) {
        const uint64_t t = uint64_t(1) << g.tgt[0];
        for (uint64_t i = 0; i < N; i++) {
            if ((i & t) || !controls_on(g, i)) continue;
            const cd a = v[i], b = v[i | t];
            v[i] = m(0, 0, 2) * a + m(0, 1, 2) * b;
            v[i | t] = m(1, 0, 2) * a + m(1, 1, 2) * b;
        }
        return;
    }
    const uint64_t ta = uint64_t(1) << g.tgt[0], tb = uint64_t(1) << g.tgt[1];
    for (uint64_t i = 0; i < N; i++) {
        if ((i & ta) || (i & tb) || !controls_on(g, i)) continue;
        const uint64_t idx[4] = {i, i | tb, i | ta, i | ta | tb};
        cd x[4], y[4];
        for (int r = 0; r < 4; r++) x[r] = v[idx[r]];
        for (int r = 0; r < 4; r++) {
            y[r] = 0;
            for (int c = 0; c < 4; c++) y[r] += m(r, c, 4) * x[c];
        }
        for (int r = 0; r < 4; r++) v[idx[r]] = y[r];
    }
}

// e^{i a} RZ(b) RY(c) RZ(d) as a 2x2 (re/im interleaved, row-major)
static void random_unitary(std::mt19937_64 &gen, double *m) {
    std::uniform_real_distribution<double> ang(-3.1, 3.1);
    const double a = ang(gen), b = ang(gen), c = ang(gen), d = ang(gen);
    const cd u[4] = {std::polar(std::cos(c / 2), a - b / 2 - d / 2), -std::polar(std::sin(c / 2), a - b / 2 + d / 2),
                     std::polar(std::sin(c / 2), a + b / 2 - d / 2), std::polar(std::cos(c / 2), a + b / 2 + d / 2)};
    for (int e = 0; e < 4; e++) {
        m[2 * e] = u[e].real();
        m[2 * e + 1] = u[e].imag();
    }
}

static size_t launches(size_t records) { return (records + lgpu::kFusedMaxGates - 1) / lgpu::kFusedMaxGates; }

static size_t real_records(const std::vector<lgpu_fused_gate_t> &f, const std::vector<char> &internal) {
    size_t r = 0;
    for (size_t i = 0; i < f.size(); i++)
        r += !internal[i] && f[i].ntgt == 1 && f[i].m[1] == 0 && f[i].m[3] == 0 && f[i].m[5] == 0 && f[i].m[7] == 0 &&
             f[i].m[0] != 0 && f[i].m[2] != 0 && f[i].m[4] != 0 && f[i].m[6] != 0;
    return r;
}

// split_dense_1q on its edge cases: structured and non-unitary matrices are
// not split; unitaries with tiny off-diagonal or diagonal entries, and with
// controls, split into parts whose product is the matrix within 1e-13, the
// middle part real and the outer ones diagonal.
static void split_edge_cases() {
    auto mk = [](const cd (&u)[4]) {
        lgpu_fused_gate_t g{};
        g.ntgt = 1;
        g.tgt[0] = 2;
        for (int e = 0; e < 4; e++) {
            g.m[2 * e] = u[e].real();
            g.m[2 * e + 1] = u[e].imag();
        }
        return g;
    };
    lgpu_fused_gate_t f[3];
    const double s = 1 / std::sqrt(2.0);
    const cd diag[4] = {std::polar(1.0, 0.3), 0, 0, std::polar(1.0, -0.3)};
    const cd anti[4] = {0, cd(0, -1), cd(0, 1), 0};
    const cd real[4] = {s, -s, s, s};
    const cd rx[4] = {std::cos(0.4), cd(0, -std::sin(0.4)), cd(0, -std::sin(0.4)), std::cos(0.4)};
    const cd nonu[4] = {cd(1, 1), cd(0.5, 0), cd(0, 0.5), cd(2, 0)};
    for (const auto *u : {&diag, &anti, &real, &rx, &nonu})
        if (lgpu::split_dense_1q(mk(*u), f)) fail("structured or non-unitary matrix split", -1, 0);
    for (double th : {1e-9, 1e-4, 0.7, 3.1415926, 3.14159265358979}) {
        // Rot(phi, th, om) with small or near-pi theta, and a control
        const double ph = 0.37, om = -1.21;
        const cd u[4] = {std::polar(std::cos(th / 2), -(ph + om) / 2), -std::polar(std::sin(th / 2), (ph - om) / 2),
                         std::polar(std::sin(th / 2), -(ph - om) / 2), std::polar(std::cos(th / 2), (ph + om) / 2)};
        lgpu_fused_gate_t g = mk(u);
        g.nctrl = 1;
        g.ctrl[0] = 5;
        g.ctrl_val[0] = 1;
        if (!lgpu::split_dense_1q(g, f)) {
            fail("dense unitary not split", -1, th);
            continue;
        }
        auto m = [](const lgpu_fused_gate_t &x, int e) { return cd(x.m[2 * e], x.m[2 * e + 1]); };
        for (int k = 0; k < 3; k++)
            if (f[k].nctrl != 1 || f[k].ctrl[0] != 5 || f[k].tgt[0] != 2) fail("split part lost its wires", -1, k);
        if (m(f[0], 1) != 0.0 || m(f[0], 2) != 0.0 || m(f[2], 1) != 0.0 || m(f[2], 2) != 0.0)
            fail("outer split part not diagonal", -1, th);
        for (int e = 0; e < 4; e++)
            if (f[1].m[2 * e + 1] != 0.0) fail("middle split part not real", -1, th);
        // product D_L R D_R
        cd q[4];
        for (int r = 0; r < 2; r++)
            for (int c = 0; c < 2; c++) q[2 * r + c] = m(f[2], 3 * r) * m(f[1], 2 * r + c) * m(f[0], 3 * c);
        for (int e = 0; e < 4; e++)
            if (std::abs(q[e] - u[e]) > 1e-13) fail("split product differs", -1, std::abs(q[e] - u[e]));
    }
}

int main() {
    split_edge_cases();
    std::mt19937_64 gen(11);
    std::normal_distribution<double> nd;
    const int n = 8, k = 6;  // tile = bits 0..5; bits 6, 7 outside
    std::vector<int> pos(n, -1);
    for (int q = 0; q < k; q++) pos[size_t(q)] = q;
    long tables = 0, folded_gates = 0, gates_total = 0, split_kept = 0;
    for (int trial = 0; trial < 600; trial++) {
        const bool layered = trial >= 400;  // dense unitaries on every tile bit, then CNOTs
        const int cnt = layered ? 3 * (k + 3) : 1 + int(gen() % 40);
        std::vector<lgpu_fused_gate_t> g(static_cast<size_t>(cnt));
        for (int gi = 0; gi < cnt && layered; gi++) {
            auto &x = g[size_t(gi)];
            x = lgpu_fused_gate_t{};
            x.ntgt = 1;
            const int r = gi % (k + 3);
            if (r < k) {
                x.tgt[0] = r;
                random_unitary(gen, x.m);
            } else {  // CNOT
                x.tgt[0] = int(gen() % k);
                do x.ctrl[0] = int(gen() % k); while (x.ctrl[0] == x.tgt[0]);
                x.ctrl_val[0] = 1;
                x.nctrl = 1;
                x.m[2] = x.m[4] = 1.0;
            }
        }
        for (auto &x : g) {
            if (layered) break;
            x = lgpu_fused_gate_t{};
            const bool two = gen() % 6 == 0;
            x.ntgt = two ? 2 : 1;
            x.tgt[0] = int(gen() % k);
            if (two) do x.tgt[1] = int(gen() % k); while (x.tgt[1] == x.tgt[0]);
            const int nc = int(gen() % 3);
            for (int c = 0; c < nc; c++) {
                int b;
                bool ok;
                do {
                    b = int(gen() % n);
                    ok = b != x.tgt[0] && (!two || b != x.tgt[1]);
                    for (int j = 0; j < x.nctrl; j++) ok = ok && x.ctrl[j] != b;
                } while (!ok);
                x.ctrl[x.nctrl] = b;
                x.ctrl_val[x.nctrl] = int(gen() % 2);
                x.nctrl++;
            }
            const int d = two ? 4 : 2;
            if (!two && gen() % 3 == 0) {  // a dense unitary (split candidate)
                random_unitary(gen, x.m);
                continue;
            }
            const bool diag = !two && gen() % 2 == 0;
            const bool sign = diag && gen() % 4 == 0;  // diag(+-1, +-1): stays a sign flip
            for (int r = 0; r < d; r++)
                for (int c = 0; c < d; c++) {
                    const bool zero = diag && r != c;
                    x.m[2 * (r * d + c)] = zero ? 0.0 : (sign ? (gen() % 2 ? 1.0 : -1.0) : nd(gen));
                    x.m[2 * (r * d + c) + 1] = zero || sign ? 0.0 : nd(gen);
                }
        }
        size_t plain_records = 0;
        for (int split = 0; split < 2; split++) {
        std::vector<char> internal;
        const auto f = lgpu::fold_diagonal_gates(g.data(), uint32_t(cnt), pos, internal, split != 0);
        if (split == 0) plain_records = f.size();
        else if (launches(f.size()) > launches(plain_records)) fail("splits add a launch", trial, double(f.size()));
        if (split && layered) split_kept += long(real_records(f, internal));
        if (internal.size() != f.size()) fail("flag count", trial, double(internal.size()));
        for (size_t i = 0; i < f.size(); i++) {
            const bool tab = internal[i] != 0;
            if (tab != (f[i].ntgt == lgpu::kDiagTableMark)) fail("flag of a record", trial, double(i));
            if (tab) {
                tables++;
                if (f[i].nctrl < 1 || f[i].nctrl > lgpu::kDiagTableBits) fail("table size", trial, f[i].nctrl);
                for (int b = 0; b < f[i].nctrl; b++)
                    if (pos[size_t(f[i].ctrl[b])] < 0) fail("table bit outside the tile", trial, f[i].ctrl[b]);
                for (int b = 1; b < f[i].nctrl; b++)
                    if (pos[size_t(f[i].ctrl[b])] <= pos[size_t(f[i].ctrl[b - 1])]) fail("table bit order", trial, b);
            }
        }
        {  // every sign-diagonal gate of the block is still there
            auto is_sign = [](const lgpu_fused_gate_t &x) {
                auto pm1 = [](double v) { return v == 1.0 || v == -1.0; };
                return x.ntgt == 1 && x.m[2] == 0.0 && x.m[3] == 0.0 && x.m[4] == 0.0 && x.m[5] == 0.0 &&
                       pm1(x.m[0]) && x.m[1] == 0.0 && pm1(x.m[6]) && x.m[7] == 0.0;
            };
            long before = 0, after = 0;
            for (const auto &x : g) before += is_sign(x);
            for (size_t i = 0; i < f.size(); i++) after += !internal[i] && is_sign(f[i]);
            if (after < before || (!split && before != after))
                fail("sign-diagonal gate folded", trial, double(before - after));
        }
        if (!split) {
            gates_total += cnt;
            folded_gates += cnt - long(f.size());
        }
        for (int rep = 0; rep < 2; rep++) {
            std::vector<cd> a(size_t(1) << n), b;
            for (auto &z : a) z = cd(nd(gen), nd(gen));
            b = a;
            for (const auto &x : g) apply(a, x, false);
            for (size_t i = 0; i < f.size(); i++) apply(b, f[i], internal[i] != 0);
            double err = 0, scale = 1e-300;
            for (size_t i = 0; i < a.size(); i++) {
                err = std::max(err, std::abs(a[i] - b[i]));
                scale = std::max(scale, std::abs(a[i]));
            }
            if (err > 1e-12 * scale) fail("state differs", trial, err / scale);
        }
        }
    }
    if (tables == 0) fail("no table formed", 0, 0);
    if (split_kept == 0) fail("no split kept", 0, 0);
    std::printf("blocks 600 gates %ld tables %ld gates folded away %ld real bodies in split layers %ld bad %ld\n",
                gates_total, tables, folded_gates, split_kept, bad);
    return bad == 0 ? 0 : 1;
}
