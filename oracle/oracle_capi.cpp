// ORACLE — test infrastructure only.  Flat extern "C" entry points over
// sv_oracle.hpp so that the Python test-suite and the CPU-baseline leg of the
// benchmark can drive the CPU restatement through ctypes.  All states are
// interleaved complex128 arrays of 2^n amplitudes (wire w <-> bit n-1-w).
#include "sv_oracle.hpp"

#include <cstring>
#include <sstream>

namespace {
thread_local std::string g_err;

using namespace oracle;

std::vector<std::string> split_names(const char *names, int64_t count) {
    std::vector<std::string> out;
    std::string cur;
    for (const char *p = names; *p; ++p) {
        if (*p == '\n') {
            out.push_back(cur);
            cur.clear();
        } else {
            cur.push_back(*p);
        }
    }
    if (!cur.empty() || int64_t(out.size()) < count) out.push_back(cur);
    if (int64_t(out.size()) != count) throw OracleError("name count mismatch");
    return out;
}

std::vector<cd> as_state(const double *s, int n) {
    const size_t N = size_t(1) << n;
    std::vector<cd> v(N);
    std::memcpy(static_cast<void *>(v.data()), s, N * sizeof(cd));
    return v;
}

Mat read_mat(const int64_t *off, const double *mats, int64_t i) {
    Mat m;
    if (!off) return m;
    for (int64_t e = off[i]; e < off[i + 1]; e++) m.emplace_back(mats[2 * e], mats[2 * e + 1]);
    return m;
}

std::vector<Op> read_ops(int nops, const char *names, const int64_t *wire_off, const int64_t *wires,
                         const int64_t *par_off, const double *params, const uint8_t *inverses,
                         const int64_t *mat_off, const double *mats) {
    const auto nm = split_names(names, nops);
    std::vector<Op> ops(static_cast<size_t>(nops));
    for (int i = 0; i < nops; i++) {
        Op &op = ops[size_t(i)];
        op.name = nm[size_t(i)];
        for (int64_t k = wire_off[i]; k < wire_off[i + 1]; k++) op.wires.push_back(int(wires[k]));
        for (int64_t k = par_off[i]; k < par_off[i + 1]; k++) op.params.push_back(params[k]);
        op.inverse = inverses ? inverses[i] != 0 : false;
        op.matrix = read_mat(mat_off, mats, i);
    }
    return ops;
}

template <class F> int guarded(F &&f) {
    try {
        f();
        return 0;
    } catch (const std::exception &e) {
        g_err = e.what();
        return 1;
    }
}
} // namespace

extern "C" {

const char *oracle_last_error(void) { return g_err.c_str(); }

void oracle_set_rot_quirk(int on) { oracle::rot_adjoint_reference_quirk() = (on != 0); }

int oracle_apply_ops(double *state, int n, int nops, const char *names, const int64_t *wire_off,
                     const int64_t *wires, const int64_t *par_off, const double *params,
                     const uint8_t *inverses, const int64_t *mat_off, const double *mats) {
    return guarded([&] {
        auto ops = read_ops(nops, names, wire_off, wires, par_off, params, inverses, mat_off, mats);
        auto sv = as_state(state, n);
        for (const auto &op : ops)
            apply_operation(sv, n, op.name, op.wires, op.inverse, op.params, op.matrix);
        std::memcpy(state, static_cast<const void *>(sv.data()), sv.size() * sizeof(cd));
    });
}

// One dense 2x2 gate on `wire` applied in place (CPU baseline of the
// single-gate workload; same loop structure as apply_matrix).
int oracle_apply_1q_inplace(double *state, int n, int wire, const double *mat4) {
    return guarded([&] {
        cd *a = reinterpret_cast<cd *>(state);
        const cd m00(mat4[0], mat4[1]), m01(mat4[2], mat4[3]), m10(mat4[4], mat4[5]),
            m11(mat4[6], mat4[7]);
        const int b = bit_of_wire(n, wire);
        const int64_t half = int64_t(1) << (n - 1);
        const uint64_t lo = (uint64_t(1) << b) - 1;
#pragma omp parallel for schedule(static)
        for (int64_t g = 0; g < half; g++) {
            const uint64_t i0 = ((uint64_t(g) >> b) << (b + 1)) | (uint64_t(g) & lo);
            const uint64_t i1 = i0 | (uint64_t(1) << b);
            const cd x = a[i0], y = a[i1];
            a[i0] = m00 * x + m01 * y;
            a[i1] = m10 * x + m11 * y;
        }
    });
}

int oracle_expval_matrix(const double *state, int n, const int64_t *wires, int k,
                         const double *mat, double *out2) {
    return guarded([&] {
        auto sv = as_state(state, n);
        std::vector<int> w(wires, wires + k);
        Mat m;
        for (int64_t e = 0; e < (int64_t(1) << (2 * k)); e++) m.emplace_back(mat[2 * e], mat[2 * e + 1]);
        const cd r = expval_matrix(sv, n, m, w);
        out2[0] = r.real();
        out2[1] = r.imag();
    });
}

int oracle_expval_pauli_words(const double *state, int n, int nwords, const char *words,
                              const int64_t *wire_off, const int64_t *wires,
                              const double *coeffs, double *out) {
    return guarded([&] {
        auto sv = as_state(state, n);
        const auto w = split_names(words, nwords);
        std::vector<std::vector<int>> ww(static_cast<size_t>(nwords));
        std::vector<cd> c(static_cast<size_t>(nwords));
        for (int t = 0; t < nwords; t++) {
            for (int64_t k = wire_off[t]; k < wire_off[t + 1]; k++) ww[size_t(t)].push_back(int(wires[k]));
            if (ww[size_t(t)].size() != w[size_t(t)].size()) throw OracleError("word/wire length mismatch");
            c[size_t(t)] = cd(coeffs[2 * t], coeffs[2 * t + 1]);
        }
        *out = expval_pauli_words(sv, n, w, ww, c);
    });
}

int oracle_probs(const double *state, int n, const int64_t *wires, int k, double *out) {
    return guarded([&] {
        auto sv = as_state(state, n);
        std::vector<int> w(wires, wires + k);
        auto p = probability(sv, n, w);
        std::memcpy(out, p.data(), p.size() * sizeof(double));
    });
}

int oracle_draws(uint64_t seed, int64_t shots, int float_draws, double *out) {
    return guarded([&] {
        auto r = float_draws ? sampler_draws<float>(seed, size_t(shots))
                             : sampler_draws<double>(seed, size_t(shots));
        std::memcpy(out, r.data(), r.size() * sizeof(double));
    });
}

int oracle_sample(const double *state, int n, uint64_t seed, int64_t shots, int float_draws,
                  uint64_t *out_idx) {
    return guarded([&] {
        auto sv = as_state(state, n);
        auto r = float_draws ? sampler_draws<float>(seed, size_t(shots))
                             : sampler_draws<double>(seed, size_t(shots));
        auto idx = sample_indices(sv, n, r);
        std::memcpy(out_idx, idx.data(), idx.size() * sizeof(uint64_t));
    });
}

int oracle_sample_from_draws(const double *state, int n, const double *draws, int64_t shots,
                             uint64_t *out_idx) {
    return guarded([&] {
        auto sv = as_state(state, n);
        std::vector<double> r(draws, draws + shots);
        auto idx = sample_indices(sv, n, r);
        std::memcpy(out_idx, idx.data(), idx.size() * sizeof(uint64_t));
    });
}

int oracle_apply_observable(double *state, int n, int nterms, const double *term_coeff,
                            int is_ham, const int64_t *term_factor_off, const char *factor_names,
                            const int64_t *factor_wire_off, const int64_t *factor_wires,
                            const int64_t *factor_mat_off, const double *factor_mats) {
    return guarded([&] {
        Observable ob;
        ob.is_hamiltonian = is_ham != 0;
        const int64_t nf = term_factor_off[nterms];
        const auto fn = split_names(factor_names, nf);
        for (int t = 0; t < nterms; t++) {
            Term term;
            term.coeff = term_coeff[t];
            for (int64_t f = term_factor_off[t]; f < term_factor_off[t + 1]; f++) {
                Factor fac;
                fac.name = fn[size_t(f)];
                for (int64_t k = factor_wire_off[f]; k < factor_wire_off[f + 1]; k++)
                    fac.wires.push_back(int(factor_wires[k]));
                fac.matrix = read_mat(factor_mat_off, factor_mats, f);
                term.factors.push_back(fac);
            }
            ob.terms.push_back(term);
        }
        auto sv = as_state(state, n);
        apply_observable(sv, n, ob);
        std::memcpy(state, static_cast<const void *>(sv.data()), sv.size() * sizeof(cd));
    });
}

// Observables are encoded as: obs k owns terms [obs_term_off[k], obs_term_off[k+1]);
// term t owns factors [term_factor_off[t], term_factor_off[t+1]).
int oracle_adjoint(const double *final_state, int n, int nops, const char *names,
                   const int64_t *wire_off, const int64_t *wires, const int64_t *par_off,
                   const double *params, const uint8_t *inverses, const int64_t *mat_off,
                   const double *mats, int nobs, const int64_t *obs_term_off,
                   const uint8_t *obs_is_ham, const double *term_coeff,
                   const int64_t *term_factor_off, const char *factor_names,
                   const int64_t *factor_wire_off, const int64_t *factor_wires,
                   const int64_t *factor_mat_off, const double *factor_mats, int64_t ntp,
                   const int64_t *tp, double *jac_out) {
    return guarded([&] {
        auto ops = read_ops(nops, names, wire_off, wires, par_off, params, inverses, mat_off, mats);
        const int64_t nterms = obs_term_off[nobs];
        const int64_t nf = term_factor_off[nterms];
        const auto fn = split_names(factor_names, nf);
        std::vector<Observable> obs(static_cast<size_t>(nobs));
        for (int k = 0; k < nobs; k++) {
            obs[size_t(k)].is_hamiltonian = obs_is_ham[k] != 0;
            for (int64_t t = obs_term_off[k]; t < obs_term_off[k + 1]; t++) {
                Term term;
                term.coeff = term_coeff[t];
                for (int64_t f = term_factor_off[t]; f < term_factor_off[t + 1]; f++) {
                    Factor fac;
                    fac.name = fn[size_t(f)];
                    for (int64_t q = factor_wire_off[f]; q < factor_wire_off[f + 1]; q++)
                        fac.wires.push_back(int(factor_wires[q]));
                    fac.matrix = read_mat(factor_mat_off, factor_mats, f);
                    term.factors.push_back(fac);
                }
                obs[size_t(k)].terms.push_back(term);
            }
        }
        std::vector<size_t> tps(tp, tp + ntp);
        auto sv = as_state(final_state, n);
        auto jac = adjoint_jacobian(sv, n, obs, ops, tps);
        for (int k = 0; k < nobs; k++)
            for (int64_t p = 0; p < ntp; p++) jac_out[k * ntp + p] = jac[size_t(k)][size_t(p)];
    });
}

int oracle_expval_sparse(const double *state, int n, const int64_t *offsets, int64_t nrows,
                         const int64_t *cols, const double *vals, double *out) {
    return guarded([&] {
        auto sv = as_state(state, n);
        if (nrows != (int64_t(1) << n)) throw OracleError("sparse matrix rows must equal 2^n");
        *out = expval_sparse(sv, offsets, nrows, cols, reinterpret_cast<const cd *>(vals));
    });
}

} // extern "C"
