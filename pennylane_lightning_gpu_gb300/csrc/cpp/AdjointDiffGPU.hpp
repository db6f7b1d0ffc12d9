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
// column stays on the device until one copy at the end.
#pragma once

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

        size_t trainableParamNumber = tp_size - 1;
        size_t current_param_idx = num_param_ops - 1;
        auto tp_it = trainableParams.rbegin();
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

        for (int op_idx = static_cast<int>(ops_name.size() - 1); op_idx >= 0; op_idx--) {
            PL_ABORT_IF(ops.getOpsParams()[size_t(op_idx)].size() > 1,
                        "The operation is not supported using the adjoint differentiation method");
            const std::string &name = ops_name[size_t(op_idx)];
            if ((name == "QubitStateVector") || (name == "StatePrep") || (name == "BasisState")) continue;
            if (tp_it == tp_rend) break;  // All done

            const bool inv = ops.getOpsInverses()[size_t(op_idx)];
            const auto &wires = ops.getOpsWires()[size_t(op_idx)];
            Engine::GateDesc udag = lower(lambda, ops, size_t(op_idx), !inv);
            std::vector<int> ubits;
            std::vector<cd> umat;
            const bool fusable = Engine::dense_on_bits(udag, ubits, umat, 4);

            bool want_grad = false;
            if (ops.hasParams(size_t(op_idx))) {
                if (current_param_idx == *tp_it) want_grad = true;
            }
            if (want_grad) {
                std::vector<cd> g;
                double scale = 0;
                std::vector<int> gbits;
                for (size_t w : wires) gbits.push_back(Engine::bit_of(n, w));
                const bool has_gen = Engine::generator_of(name, gbits.size(), g, scale);
                PL_ABORT_IF_NOT(has_gen, ("The operation " + name +
                                          " is not supported using the adjoint differentiation method")
                                             .c_str());
                col_scale[trainableParamNumber] = scale * (inv ? -1.0 : 1.0);
                double *out = jac_dev.getData() + trainableParamNumber * K;
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
                trainableParamNumber--;
                ++tp_it;
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
            if (ops.hasParams(size_t(op_idx))) current_param_idx--;
        }
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
