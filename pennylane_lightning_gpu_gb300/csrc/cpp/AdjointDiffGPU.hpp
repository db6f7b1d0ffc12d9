// AdjointJacobianGPU<T>: the adjoint-Jacobian reverse sweep (reference
// src/algorithms/AdjointDiffGPU.hpp:49-597).
//
// Same algorithm and bookkeeping as the reference: K bra states O_k|psi>, a
// reverse walk over the operations that skips state preparations, aborts on
// multi-parameter ops, and fills jac[k][p] = -2 * s * Im<bra_k|G|lambda> with
// the reference's generator scale factors s (sign flipped for inverted ops).
// Per operation the engine issues ONE fused launch (lgpu_adjoint_step) that
// reads lambda and the K bras once, forms the generator expectations, and
// applies U^dag to all of them; mu is never materialised and the Jacobian
// column stays on the device until one copy at the end.  Runs of 1-target
// operations whose targets fit a shared-memory tile take one pass for the
// whole run (lgpu_adjoint_block_ff); a run may take an operation ahead of
// operations it leaves behind when they share no wire (the operations and
// their generators then commute), so each operation's Jacobian column is
// fixed up front instead of by the walk's counters.
#pragma once

#include <cstdlib>
#include <memory>
#include <vector>

#include "JacobianData.hpp"
#include "ObservablesGPU.hpp"

namespace Pennylane::Algorithms {

template <class T = double> class AdjointJacobianGPU {
  private:
    using CFP_t = decltype(cuUtil::getCudaType(T{}));
    using SV = StateVectorCudaManaged<T>;
    using cd = std::complex<double>;

  public:
    AdjointJacobianGPU() = default;

    auto createOpsData(const std::vector<std::string> &ops_name, const std::vector<std::vector<T>> &ops_params,
                       const std::vector<std::vector<size_t>> &ops_wires, const std::vector<bool> &ops_inverses,
                       const std::vector<std::vector<std::complex<T>>> &ops_matrices = {{}}) -> OpsData<SV> {
        return {ops_name, ops_params, ops_wires, ops_inverses, ops_matrices};
    }

    // Apply every operation of `opsData` to `sv` (AdjointDiffGPU.hpp:172-181).
    inline void applyOperations(SV &sv, const OpsData<SV> &opsData, bool adj = false) {
        for (size_t op_idx = 0; op_idx < opsData.getOpsName().size(); op_idx++)
            applyOp(sv, opsData, op_idx, adj ^ opsData.getOpsInverses()[op_idx]);
    }
    // Apply the adjoint of operation op_idx (AdjointDiffGPU.hpp:190-200).
    inline void applyOperationAdj(SV &sv, const OpsData<SV> &ops, size_t op_idx) {
        applyOp(sv, ops, op_idx, !ops.getOpsInverses()[op_idx]);
    }
    inline void applyObservable(SV &sv, ObservableGPU<T> &observable) { observable.applyInPlace(sv); }
    inline void applyObservables(std::vector<SV> &states, const SV &reference_state,
                                 const std::vector<std::shared_ptr<ObservableGPU<T>>> &observables) {
        for (size_t k = 0; k < observables.size(); k++) {
            states[k].updateData(reference_state);
            observables[k]->applyInPlace(states[k]);
        }
    }
    inline void applyOperationsAdj(std::vector<SV> &states, const OpsData<SV> &ops, size_t op_idx) {
        for (auto &s : states) applyOperationAdj(s, ops, op_idx);
    }
    // Applies the generator of op `opName` on wires and returns its scale
    // factor (AdjointDiffGPU.hpp:210-216).
    inline T applyGenerator(SV &sv, const std::string &opName, const std::vector<size_t> &wires, const bool adj) {
        return static_cast<T>(sv.applyGeneratorOf(opName, wires, adj));
    }

    void adjointJacobian(const CFP_t *ref_data, std::size_t length, std::vector<std::vector<T>> &jac,
                         const std::vector<std::shared_ptr<ObservableGPU<T>>> &obs, const OpsData<SV> &ops,
                         const std::vector<size_t> &trainableParams, bool apply_operations = false,
                         CUDA::DevTag<int> dev_tag = {0, 0}) {
        PL_ABORT_IF(trainableParams.empty(), "No trainable parameters provided.");
        const std::vector<std::string> &ops_name = ops.getOpsName();
        const size_t num_observables = obs.size();
        const size_t tp_size = trainableParams.size();
        const size_t num_param_ops = ops.getNumParOps();
        PL_ABORT_IF(jac.size() < num_observables, "Jacobian has too few rows");
        for (auto &row : jac) PL_ABORT_IF(row.size() < tp_size, "Jacobian has too few columns");

        const auto tp_rend = trainableParams.rend();

        CUDA::DevTag<int> dt_local(std::move(dev_tag));
        dt_local.refresh();
        SV lambda(ref_data, length, dt_local);
        if (apply_operations) applyOperations(lambda, ops);
        const uint32_t n = uint32_t(lambda.getNumQubits());

        std::vector<SV> H_lambda;
        H_lambda.reserve(num_observables);
        for (size_t k = 0; k < num_observables; k++) H_lambda.emplace_back(lambda.getNumQubits(), dt_local, true);
        applyObservables(H_lambda, lambda, obs);
        std::vector<void *> bra_ptrs(num_observables);
        for (size_t k = 0; k < num_observables; k++) bra_ptrs[k] = H_lambda[k].getData();

        // Device-resident Jacobian columns: [tp_size][num_observables].
        const size_t K = std::max<size_t>(num_observables, 1);
        CUDA::DataBuffer<double, int> jac_dev(tp_size * K, dt_local, true);
        jac_dev.zeroInit();
        std::vector<double> col_scale(tp_size, 0.0);
        std::unique_ptr<SV> mu;  // only for operations the fused step cannot take

        // States that fit in shared memory: the whole sweep in one launch
        // when every operation acts on at most two bits.
        if (num_observables > 0 && n <= lgpu_adjoint_sweep_max_qubits(SV::dt())) {
            std::vector<lgpu_adj_op_t> sweep;
            std::vector<double> scales(tp_size, 0.0);
            bool ok = true;
            size_t tpn = tp_size - 1, cpi = num_param_ops - 1;
            auto it = trainableParams.rbegin();
            for (int op_idx = static_cast<int>(ops_name.size() - 1); op_idx >= 0 && ok; op_idx--) {
                PL_ABORT_IF(ops.getOpsParams()[size_t(op_idx)].size() > 1,
                            "The operation is not supported using the adjoint differentiation method");
                const std::string &name = ops_name[size_t(op_idx)];
                if ((name == "QubitStateVector") || (name == "StatePrep") || (name == "BasisState")) continue;
                if (it == tp_rend) break;
                const bool inv = ops.getOpsInverses()[size_t(op_idx)];
                const auto &wires = ops.getOpsWires()[size_t(op_idx)];
                Engine::GateDesc udag = lower(lambda, ops, size_t(op_idx), !inv);
                std::vector<int> ubits;
                std::vector<cd> umat;
                lgpu_adj_op_t a{};
                a.col = -1;
                if (udag.kind == Engine::GateDesc::IDENTITY) {
                    a.nu = 1;
                    a.ubits[0] = Engine::bit_of(n, wires.empty() ? 0 : wires[0]);
                    a.u[0] = a.u[6] = 1.0;
                } else if (Engine::dense_on_bits(udag, ubits, umat, 2)) {
                    a.nu = int32_t(ubits.size());
                    for (size_t q = 0; q < ubits.size(); q++) a.ubits[q] = ubits[q];
                    for (size_t e = 0; e < umat.size(); e++) {
                        a.u[2 * e] = umat[e].real();
                        a.u[2 * e + 1] = umat[e].imag();
                    }
                } else {
                    ok = false;
                    break;
                }
                if (ops.hasParams(size_t(op_idx)) && cpi == *it) {
                    std::vector<cd> g;
                    double scale = 0;
                    PL_ABORT_IF_NOT(Engine::generator_of(name, wires.size(), g, scale),
                                    ("The operation " + name +
                                     " is not supported using the adjoint differentiation method")
                                        .c_str());
                    if (wires.size() > 2) {
                        ok = false;
                        break;
                    }
                    a.ng = int32_t(wires.size());
                    for (size_t q = 0; q < wires.size(); q++) a.gbits[q] = Engine::bit_of(n, wires[q]);
                    for (size_t e = 0; e < g.size(); e++) {
                        a.g[2 * e] = g[e].real();
                        a.g[2 * e + 1] = g[e].imag();
                    }
                    a.col = int32_t(tpn);
                    scales[tpn] = scale * (inv ? -1.0 : 1.0);
                    tpn--;
                    ++it;
                }
                if (ops.hasParams(size_t(op_idx))) cpi--;
                sweep.push_back(a);
            }
            if (ok) {
                PL_LGPU_IS_SUCCESS(lgpu_adjoint_sweep_small(lambda.ctx(), lambda.getData(), bra_ptrs.data(),
                                                            uint32_t(num_observables), n, SV::dt(), sweep.data(),
                                                            uint32_t(sweep.size()), jac_dev.getData(),
                                                            lambda.lstream()));
                std::vector<double> host(tp_size * K);
                jac_dev.CopyGpuDataToHost(host.data(), host.size(), false);
                for (size_t p = 0; p < tp_size; p++)
                    for (size_t k = 0; k < num_observables; k++)
                        jac[k][p] = static_cast<T>(-2.0 * scales[p] * host[p * K + k]);
                return;
            }
        }

        const bool blocks = num_observables >= 1 && blocks_enabled();
        std::unique_ptr<SV> lam0;  // lambda before a block, when the bras run in pairs
        // complex128: between consecutive blocks lambda and the bras stay in
        // float-float form (lgpu_state_ff); any other operation gets them back
        // as complex128 first
        const bool ff_ok = SV::dt() == LGPU_C128;
        bool in_ff = false;
        auto leave_ff = [&]() {
            if (!in_ff) return;
            PL_LGPU_IS_SUCCESS(lgpu_state_ff(lambda.getData(), n, 0, lambda.lstream()));
            for (size_t k = 0; k < num_observables; k++)
                PL_LGPU_IS_SUCCESS(lgpu_state_ff(bra_ptrs[k], n, 0, lambda.lstream()));
            in_ff = false;
        };
        // The Jacobian column of every operation (-1: no trainable parameter),
        // as the reference's reverse counters assign them.
        const size_t nops = ops_name.size();
        std::vector<int> col(nops, -1);
        size_t cols_left = 0;
        {
            size_t pi = 0, t = 0;
            for (size_t j = 0; j < nops; j++) {
                if (!ops.hasParams(j)) continue;
                while (t < tp_size && trainableParams[t] < pi) t++;
                if (t < tp_size && trainableParams[t] == pi) {
                    col[j] = int(t);
                    cols_left++;
                }
                pi++;
            }
        }
        auto is_prep = [&](size_t j) {
            const std::string &nm = ops_name[j];
            return nm == "QubitStateVector" || nm == "StatePrep" || nm == "BasisState";
        };
        auto wire_bits = [&](size_t j) {
            uint64_t b = 0;
            for (size_t w : ops.getOpsWires()[j]) b |= uint64_t(1) << Engine::bit_of(n, w);
            return b;
        };
        std::vector<char> done(nops, 0);
        int op_idx = static_cast<int>(nops) - 1;
        while (op_idx >= 0) {
            if (done[size_t(op_idx)]) {
                op_idx--;
                continue;
            }
            PL_ABORT_IF(ops.getOpsParams()[size_t(op_idx)].size() > 1,
                        "The operation is not supported using the adjoint differentiation method");
            const std::string &name = ops_name[size_t(op_idx)];
            if (is_prep(size_t(op_idx))) {
                op_idx--;
                continue;
            }
            if (cols_left == 0) break;  // All done

            // A run of 1-target operations (with controls) whose targets fit
            // one tile: one pass over lambda and the bras for the whole run.
            // The run takes operations in reverse order; an operation that
            // cannot join (not a 1-target step, target outside the tile) is
            // left for later and blocks its wires, and a later operation joins
            // only if it shares no wire with any operation left behind (so it
            // commutes with them and with their generators).
            if (blocks) {
                std::vector<lgpu_adj_block_step_t> steps;
                std::vector<int> tbits, tile;
                std::vector<std::pair<size_t, double>> scales;
                std::vector<size_t> taken;
                uint64_t blocked = 0;
                const uint64_t all_bits = n >= 64 ? ~uint64_t(0) : (uint64_t(1) << n) - 1;
                int scanned = 0;
                for (int j = op_idx; j >= 0 && steps.size() < 48 && scanned < 512 && blocked != all_bits; j--) {
                    if (done[size_t(j)] || is_prep(size_t(j))) continue;
                    if (ops.getOpsParams()[size_t(j)].size() > 1) break;  // aborts when the sweep reaches it
                    scanned++;
                    const uint64_t wb = wire_bits(size_t(j));
                    if (wb & blocked) {
                        blocked |= wb;
                        continue;
                    }
                    const std::string &nj = ops_name[size_t(j)];
                    const bool invj = ops.getOpsInverses()[size_t(j)];
                    const bool grad = col[size_t(j)] >= 0;
                    lgpu_adj_block_step_t st{};
                    double scale = 0;
                    std::vector<int> trial(tbits), t2;
                    bool ok = block_step(lower(lambda, ops, size_t(j), !invj), nj, ops.getOpsWires()[size_t(j)], n,
                                         grad, st, scale);
                    if (ok) {
                        trial.push_back(st.tgt);
                        ok = Engine::tile_for(trial, 11, 5, n, t2, 6);
                    }
                    if (!ok) {
                        blocked |= wb;
                        continue;
                    }
                    tbits = trial;
                    tile = t2;
                    if (grad) {
                        st.col = int32_t(col[size_t(j)]);
                        scales.emplace_back(size_t(col[size_t(j)]), scale * (invj ? -1.0 : 1.0));
                    }
                    steps.push_back(st);
                    taken.push_back(size_t(j));
                }
                if (steps.size() >= 2) {
                    std::vector<int32_t> tb(tile.begin(), tile.end());
                    // Up to two bras per pass; more run in pairs, each pair
                    // starting from the same lambda (restored from a copy).
                    if (num_observables > 2) {
                        if (!lam0) lam0 = std::make_unique<SV>(lambda.getNumQubits(), dt_local, true);
                        lam0->updateData(lambda);
                    }
                    const uint32_t ff = ff_ok ? ((in_ff ? LGPU_FF_IN : 0u) | LGPU_FF_OUT) : 0u;
                    for (size_t b0 = 0; b0 < num_observables; b0 += 2) {
                        if (b0 > 0) lambda.updateData(*lam0);
                        const uint32_t nb = uint32_t(std::min<size_t>(2, num_observables - b0));
                        PL_LGPU_IS_SUCCESS(lgpu_adjoint_block_ff(lambda.ctx(), lambda.getData(), bra_ptrs.data() + b0,
                                                                 nb, n, SV::dt(), uint32_t(tb.size()), tb.data(),
                                                                 steps.data(), uint32_t(steps.size()),
                                                                 jac_dev.getData() + b0, uint32_t(K), ff,
                                                                 lambda.lstream()));
                    }
                    in_ff = ff_ok;
                    for (const auto &cs : scales) col_scale[cs.first] = cs.second;
                    for (size_t j : taken) done[j] = 1;
                    cols_left -= scales.size();
                    continue;  // op_idx again: it may have been left behind
                }
            }

            leave_ff();
            const bool inv = ops.getOpsInverses()[size_t(op_idx)];
            const auto &wires = ops.getOpsWires()[size_t(op_idx)];
            Engine::GateDesc udag = lower(lambda, ops, size_t(op_idx), !inv);
            std::vector<int> ubits;
            std::vector<cd> umat;
            const bool fusable = Engine::dense_on_bits(udag, ubits, umat, 4);

            const int opcol = col[size_t(op_idx)];
            if (opcol >= 0) {
                std::vector<cd> g;
                double scale = 0;
                std::vector<int> gbits;
                for (size_t w : wires) gbits.push_back(Engine::bit_of(n, w));
                const bool has_gen = Engine::generator_of(name, gbits.size(), g, scale);
                PL_ABORT_IF_NOT(has_gen, ("The operation " + name +
                                          " is not supported using the adjoint differentiation method")
                                             .c_str());
                col_scale[size_t(opcol)] = scale * (inv ? -1.0 : 1.0);
                double *out = jac_dev.getData() + size_t(opcol) * K;
                if (fusable && gbits == ubits) {
                    std::vector<int32_t> b32(ubits.begin(), ubits.end());
                    PL_LGPU_IS_SUCCESS(lgpu_adjoint_step(lambda.ctx(), lambda.getData(), bra_ptrs.data(),
                                                         uint32_t(num_observables), n, SV::dt(), uint32_t(b32.size()),
                                                         b32.data(), reinterpret_cast<const double *>(g.data()),
                                                         reinterpret_cast<const double *>(umat.data()), 1, out,
                                                         lambda.lstream()));
                } else {
                    // mu = G lambda ; out[k] = Im <bra_k|mu> ; then U^dag everywhere.
                    if (!mu) mu = std::make_unique<SV>(lambda.getNumQubits(), dt_local, true);
                    mu->updateData(lambda);
                    mu->applyGeneratorOf(name, wires, !inv);
                    for (size_t k = 0; k < num_observables; k++) {
                        PL_LGPU_IS_SUCCESS(lgpu_dot(lambda.ctx(), H_lambda[k].getData(), mu->getData(), n, SV::dt(),
                                                    dot_buf(lambda), 1, lambda.lstream()));
                        // imaginary part of the dot product -> out[k]
                        PL_LGPU_IS_SUCCESS(lgpu_memcpy(out + k, dot_buf(lambda) + 1, sizeof(double), LGPU_D2D, 1,
                                                       lambda.lstream()));
                    }
                    lambda.applyDesc(udag);
                    for (auto &b : H_lambda) b.applyDesc(udag);
                }
                cols_left--;
            } else {
                if (fusable && ubits.size() == 1) {
                    std::vector<int32_t> b32(ubits.begin(), ubits.end());
                    PL_LGPU_IS_SUCCESS(lgpu_adjoint_step(lambda.ctx(), lambda.getData(), bra_ptrs.data(),
                                                         uint32_t(num_observables), n, SV::dt(), uint32_t(b32.size()),
                                                         b32.data(), nullptr, reinterpret_cast<const double *>(umat.data()),
                                                         1, nullptr, lambda.lstream()));
                } else {
                    // no gradient here: the gate kernels (structured bodies,
                    // controls as index holes) update lambda and every bra
                    // in one launch
                    std::vector<void *> all(bra_ptrs);
                    all.push_back(lambda.getData());
                    lambda.applyDescMulti(udag, all);
                }
            }
            done[size_t(op_idx)] = 1;
            op_idx--;
        }
        leave_ff();  // lambda and the bras leave the sweep as complex128
        // One device-to-host copy of all columns.
        std::vector<double> host(tp_size * K);
        jac_dev.CopyGpuDataToHost(host.data(), host.size(), false);
        for (size_t p = 0; p < tp_size; p++)
            for (size_t k = 0; k < num_observables; k++)
                jac[k][p] = static_cast<T>(-2.0 * col_scale[p] * host[p * K + k]);
    }

    // Observable batching over devices (AdjointDiffGPU.hpp:392-473).  There is
    // one GPU, so the batch runs through the single-device sweep.
    void batchAdjointJacobian(const CFP_t *ref_data, std::size_t length, std::vector<std::vector<T>> &jac,
                              const std::vector<std::shared_ptr<ObservableGPU<T>>> &obs, const OpsData<SV> &ops,
                              const std::vector<size_t> &trainableParams, bool apply_operations = false) {
        adjointJacobian(ref_data, length, jac, obs, ops, trainableParams, apply_operations, CUDA::DevTag<int>{0, 0});
    }

  private:
    // Fused adjoint blocks are on unless LGPU_ADJOINT_BLOCKS=0.
    static bool blocks_enabled() {
        static const bool on = [] {
            const char *e = std::getenv("LGPU_ADJOINT_BLOCKS");
            return !(e && e[0] == '0');
        }();
        return on;
    }
    // The operation as a step of a fused adjoint block: U^dag a 1-target
    // gate with at most 2 controls, and (grad) its generator either a 2x2 on
    // the target of an uncontrolled 1-wire operation, or P11 (x) g on
    // (control, target) for the controlled rotations and phase.
    static bool block_step(const Engine::GateDesc &u, const std::string &name, const std::vector<size_t> &wires,
                           uint32_t n, bool grad, lgpu_adj_block_step_t &st, double &scale) {
        std::vector<cd> m2;
        if (u.kind == Engine::GateDesc::IDENTITY) {
            if (wires.size() != 1) return false;
            st.tgt = Engine::bit_of(n, wires[0]);
            m2 = {1.0, 0.0, 0.0, 1.0};
        } else {
            if (u.tgts.size() != 1 || u.ctrls.size() > 2) return false;
            st.tgt = u.tgts[0];
            if (u.kind == Engine::GateDesc::MATRIX) {
                if (u.matrix.size() != 4) return false;
                m2 = u.matrix;
            } else {
                Engine::GateDesc bare = u;
                bare.ctrls.clear();
                bare.cvals.clear();
                std::vector<int> bits;
                if (!Engine::dense_on_bits(bare, bits, m2, 1) || m2.size() != 4) return false;
            }
            st.nctrl = int32_t(u.ctrls.size());
            for (size_t c = 0; c < u.ctrls.size(); c++) {
                st.ctrl[c] = u.ctrls[c];
                st.ctrl_val[c] = u.cvals.empty() ? 1 : u.cvals[c];
            }
        }
        for (int e = 0; e < 4; e++) {
            st.u[2 * e] = m2[size_t(e)].real();
            st.u[2 * e + 1] = m2[size_t(e)].imag();
        }
        st.gen_kind = -1;
        st.col = -1;
        if (!grad) return true;
        std::vector<cd> g;
        if (!Engine::generator_of(name, wires.size(), g, scale)) return false;
        std::vector<cd> g1;
        if (wires.size() == 1 && st.nctrl == 0 && g.size() == 4) {
            g1 = g;
        } else if (wires.size() == 2 && g.size() == 16 && st.nctrl == 1 &&
                   st.ctrl[0] == Engine::bit_of(n, wires[0]) && st.ctrl_val[0] == 1 &&
                   st.tgt == Engine::bit_of(n, wires[1])) {
            for (int r = 0; r < 4; r++)
                for (int c = 0; c < 4; c++)
                    if ((r < 2 || c < 2) && g[size_t(r * 4 + c)] != cd(0.0)) return false;
            g1 = {g[10], g[11], g[14], g[15]};
        } else {
            return false;
        }
        for (int e = 0; e < 4; e++) {
            st.g[2 * e] = g1[size_t(e)].real();
            st.g[2 * e + 1] = g1[size_t(e)].imag();
        }
        st.gen_kind = 0;
        return true;
    }
    double *dot_buf(SV &sv) {
        if (!dot_buf_) dot_buf_ = std::make_unique<CUDA::DataBuffer<double, int>>(2, sv.getDataBuffer().getDevTag(), true);
        return dot_buf_->getData();
    }
    static Engine::GateDesc lower(const SV &sv, const OpsData<SV> &ops, size_t idx, bool adjoint) {
        const auto &pm = ops.getOpsParams()[idx];
        const std::vector<double> p(pm.begin(), pm.end());
        std::vector<cd> um;
        for (const auto &v : ops.getOpsMatrices()[idx]) um.emplace_back(double(v.real()), double(v.imag()));
        return Engine::lower_operation(sv.getNumQubits(), ops.getOpsName()[idx], ops.getOpsWires()[idx], adjoint, p,
                                       um);
    }
    static void applyOp(SV &sv, const OpsData<SV> &ops, size_t idx, bool adjoint) {
        sv.applyDesc(lower(sv, ops, idx, adjoint));
    }
    std::unique_ptr<CUDA::DataBuffer<double, int>> dot_buf_;
};

} // namespace Pennylane::Algorithms
