// Host test of the phase groups of the adjoint blocks
// (lgpu_adj_plan.h::plan_phase_groups).  Random runs of steps on 6 qubits:
// RZ and PhaseShift (diagonal, generators Z and P1, the groupable ones,
// with or without a gradient), RX and RY with gradients, Hadamard-like dense
// steps, CZ and controlled-RZ (diagonal with a control) and CNOT-like
// controlled steps.  Each step of the reverse sweep takes Im <bra| G |ket>
// and then applies U^dag to both states.  The planned sweep takes every
// group's overlaps before any of its U^dag, then applies them.  Checks: every
// step appears once; groups hold only groupable steps, at most max_bits (3 or
// 4) positions and max_grads gradients; the overlaps of every step and the final
// states equal those of the original order (within 1e-12) for random states.
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdio>
#include <random>
#include <vector>

#include "lgpu_adj_plan.h"

using cd = std::complex<double>;
static long bad = 0;

static void fail(const char *what, int trial, double v) {
    if (bad < 20) std::printf("bad %s (trial %d): %g\n", what, trial, v);
    bad++;
}

enum Gen { GNONE, GZ, GP1, GX, GY };

struct Step {
    int q;
    int ctrl;  // -1: none
    cd u[4];   // U^dag, row-major
    Gen gen;
};

static void apply_u(std::vector<cd> &v, const Step &s) {
    const size_t t = size_t(1) << s.q;
    for (size_t i = 0; i < v.size(); i++) {
        if (i & t) continue;
        if (s.ctrl >= 0 && !((i >> s.ctrl) & 1u)) continue;
        const cd a = v[i], b = v[i | t];
        v[i] = s.u[0] * a + s.u[1] * b;
        v[i | t] = s.u[2] * a + s.u[3] * b;
    }
}

// Im <bra| G |ket>, G on the target (uncontrolled steps only carry gradients)
static double overlap(const std::vector<cd> &bra, const std::vector<cd> &ket, const Step &s) {
    const size_t t = size_t(1) << s.q;
    cd acc = 0;
    for (size_t i = 0; i < ket.size(); i++) {
        if (i & t) continue;
        const cd k0 = ket[i], k1 = ket[i | t];
        cd g0, g1;
        switch (s.gen) {
        case GZ: g0 = k0; g1 = -k1; break;
        case GP1: g0 = 0; g1 = k1; break;
        case GX: g0 = k1; g1 = k0; break;
        case GY: g0 = cd(0, -1) * k1; g1 = cd(0, 1) * k0; break;
        default: g0 = g1 = 0; break;
        }
        acc += std::conj(bra[i]) * g0 + std::conj(bra[i | t]) * g1;
    }
    return acc.imag();
}

int main() {
    std::mt19937_64 gen(7);
    std::uniform_real_distribution<double> ang(-3.1, 3.1);
    std::normal_distribution<double> nd;
    const int n = 6;
    const int max_grads = 4;
    long groups = 0, grouped = 0, moved = 0;
    for (int trial = 0; trial < 500; trial++) {
        const int max_bits = 3 + trial % 2;  // the tables of 3 and 4 positions
        const int len = 2 + int(gen() % 46);
        std::vector<Step> st(static_cast<size_t>(len), Step{});
        std::vector<lgpu::AdjPlanStep> ps(static_cast<size_t>(len));
        for (int i = 0; i < len; i++) {
            Step &s = st[size_t(i)];
            s.q = int(gen() % n);
            s.ctrl = -1;
            s.gen = GNONE;
            const int kind = int(gen() % 10);
            const double th = ang(gen);
            const bool grad = gen() % 3 != 0;
            if (kind <= 3) {  // RZ(th)^dag
                s.u[0] = std::polar(1.0, th / 2);
                s.u[3] = std::polar(1.0, -th / 2);
                s.gen = grad ? GZ : GNONE;
            } else if (kind == 4) {  // PhaseShift(th)^dag
                s.u[0] = 1;
                s.u[3] = std::polar(1.0, -th);
                s.gen = grad ? GP1 : GNONE;
            } else if (kind == 5) {  // RY(th)^dag
                s.u[0] = s.u[3] = std::cos(th / 2);
                s.u[1] = std::sin(th / 2);
                s.u[2] = -std::sin(th / 2);
                s.gen = GY;
            } else if (kind == 6) {  // RX(th)^dag
                s.u[0] = s.u[3] = std::cos(th / 2);
                s.u[1] = s.u[2] = cd(0, std::sin(th / 2));
                s.gen = GX;
            } else if (kind == 7) {  // Hadamard-like, no gradient
                s.u[0] = s.u[1] = s.u[2] = 1 / std::sqrt(2.0);
                s.u[3] = -1 / std::sqrt(2.0);
            } else {  // controlled: CZ, controlled RZ (diagonal) or CNOT (not)
                do s.ctrl = int(gen() % n); while (s.ctrl == s.q);
                const int c = int(gen() % 3);
                if (c == 0) {
                    s.u[0] = 1;
                    s.u[3] = -1;
                } else if (c == 1) {
                    s.u[0] = std::polar(1.0, th / 2);
                    s.u[3] = std::polar(1.0, -th / 2);
                } else {
                    s.u[1] = s.u[2] = 1;
                }
            }
            const bool diag = s.u[1] == cd(0) && s.u[2] == cd(0);
            ps[size_t(i)] = lgpu::AdjPlanStep{s.q, diag && s.ctrl < 0 && (s.gen == GNONE || s.gen == GZ || s.gen == GP1),
                                              diag, s.gen != GNONE};
        }
        const auto plan = lgpu::plan_phase_groups(ps, max_bits, max_grads);
        std::vector<int> seen(size_t(len), 0);
        for (const auto &e : plan) {
            for (uint32_t i : e) seen[i]++;
            if (e.size() < 2) continue;
            groups++;
            grouped += long(e.size());
            uint64_t pm = 0;
            int ng = 0;
            for (size_t k = 0; k < e.size(); k++) {
                const uint32_t i = e[k];
                if (!ps[i].groupable) fail("step in a group not groupable", trial, i);
                pm |= uint64_t(1) << ps[i].q;
                ng += ps[i].grad ? 1 : 0;
                if (k && e[k] <= e[k - 1]) fail("group order", trial, i);
                if (k && e[k] != e[k - 1] + 1) moved++;
            }
            if (__builtin_popcountll(pm) > max_bits) fail("group positions", trial, double(pm));
            if (ng > max_grads) fail("group gradients", trial, ng);
        }
        for (int i = 0; i < len; i++)
            if (seen[size_t(i)] != 1) fail("step count", trial, i);
        // the two sweeps on random states
        std::vector<cd> k0(size_t(1) << n), b0(size_t(1) << n);
        for (auto &z : k0) z = cd(nd(gen), nd(gen));
        for (auto &z : b0) z = cd(nd(gen), nd(gen));
        std::vector<cd> ka = k0, ba = b0, kb = k0, bb = b0;
        std::vector<double> ova(size_t(len), 0), ovb(size_t(len), 0);
        for (int i = 0; i < len; i++) {
            if (st[size_t(i)].gen != GNONE) ova[size_t(i)] = overlap(ba, ka, st[size_t(i)]);
            apply_u(ka, st[size_t(i)]);
            apply_u(ba, st[size_t(i)]);
        }
        for (const auto &e : plan) {
            for (uint32_t i : e)
                if (st[i].gen != GNONE) ovb[i] = overlap(bb, kb, st[i]);
            for (uint32_t i : e) {
                apply_u(kb, st[i]);
                apply_u(bb, st[i]);
            }
        }
        double err = 0;
        for (int i = 0; i < len; i++) err = std::max(err, std::abs(ova[size_t(i)] - ovb[size_t(i)]));
        if (err > 1e-12 * double(size_t(1) << n)) fail("overlap differs", trial, err);
        double serr = 0;
        for (size_t i = 0; i < ka.size(); i++) serr = std::max({serr, std::abs(ka[i] - kb[i]), std::abs(ba[i] - bb[i])});
        if (serr > 1e-12) fail("final state differs", trial, serr);
    }
    if (groups == 0 || moved == 0) fail("no group formed across other steps", 0, double(groups));
    std::printf("runs 500 groups %ld grouped steps %ld moved %ld bad %ld\n", groups, grouped, moved, bad);
    return bad == 0 ? 0 : 1;
}
