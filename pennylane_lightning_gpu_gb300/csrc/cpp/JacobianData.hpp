// OpsData: the serialised operation list handed to the adjoint method.  The
// reference takes it from the (unvendored) pennylane-lightning
// algorithms/JacobianData.hpp; this is a restatement of its interface:
// names, params, wires, inverses and matrices per operation.
#pragma once

#include <complex>
#include <string>
#include <vector>

#include "Error.hpp"

namespace Pennylane::Algorithms {

template <class StateVectorT> class OpsData {
  public:
    using PrecisionT = typename StateVectorT::PrecisionT;
    using ComplexT = std::complex<PrecisionT>;

  private:
    size_t num_par_ops_;
    size_t num_nonpar_ops_;
    const std::vector<std::string> ops_name_;
    const std::vector<std::vector<PrecisionT>> ops_params_;
    const std::vector<std::vector<size_t>> ops_wires_;
    const std::vector<bool> ops_inverses_;
    const std::vector<std::vector<ComplexT>> ops_matrices_;

  public:
    OpsData(std::vector<std::string> ops_name, const std::vector<std::vector<PrecisionT>> &ops_params,
            std::vector<std::vector<size_t>> ops_wires, std::vector<bool> ops_inverses,
            std::vector<std::vector<ComplexT>> ops_matrices)
        : ops_name_{std::move(ops_name)}, ops_params_{ops_params}, ops_wires_{std::move(ops_wires)},
          ops_inverses_{std::move(ops_inverses)}, ops_matrices_{std::move(ops_matrices)} {
        num_par_ops_ = 0;
        for (const auto &p : ops_params) num_par_ops_ += static_cast<size_t>(!p.empty());
        num_nonpar_ops_ = ops_params.size() - num_par_ops_;
        PL_ABORT_IF(ops_name_.size() != ops_params_.size() || ops_name_.size() != ops_wires_.size() ||
                        ops_name_.size() != ops_inverses_.size() || ops_name_.size() != ops_matrices_.size(),
                    "The number of names, params, wires, inverses and matrices must be equal");
    }

    OpsData(const std::vector<std::string> &ops_name, const std::vector<std::vector<PrecisionT>> &ops_params,
            std::vector<std::vector<size_t>> ops_wires, std::vector<bool> ops_inverses)
        : OpsData(ops_name, ops_params, std::move(ops_wires), std::move(ops_inverses),
                  std::vector<std::vector<ComplexT>>(ops_name.size())) {}

    [[nodiscard]] auto getSize() const -> size_t { return ops_name_.size(); }
    [[nodiscard]] auto getOpsName() const -> const std::vector<std::string> & { return ops_name_; }
    [[nodiscard]] auto getOpsParams() const -> const std::vector<std::vector<PrecisionT>> & { return ops_params_; }
    [[nodiscard]] auto getOpsWires() const -> const std::vector<std::vector<size_t>> & { return ops_wires_; }
    [[nodiscard]] auto getOpsInverses() const -> const std::vector<bool> & { return ops_inverses_; }
    [[nodiscard]] auto getOpsMatrices() const -> const std::vector<std::vector<ComplexT>> & { return ops_matrices_; }
    [[nodiscard]] inline auto hasParams(size_t index) const -> bool { return !ops_params_[index].empty(); }
    [[nodiscard]] auto getNumParOps() const -> size_t { return num_par_ops_; }
    [[nodiscard]] auto getNumNonParOps() const -> size_t { return num_nonpar_ops_; }
    [[nodiscard]] auto getTotalNumParams() const -> size_t {
        size_t s = 0;
        for (const auto &p : ops_params_) s += p.size();
        return s;
    }
};

} // namespace Pennylane::Algorithms
