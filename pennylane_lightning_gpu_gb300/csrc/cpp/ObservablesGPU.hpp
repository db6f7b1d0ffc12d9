// Observable family used by the adjoint method (reference
// src/algorithms/ObservablesGPU.hpp:32-610): NamedObsGPU, HermitianObsGPU,
// TensorProdObsGPU, HamiltonianGPU, SparseHamiltonianGPU.  applyInPlace()
// replaces |psi> by O|psi>.  A Hamiltonian whose terms are all Pauli words is
// applied with one streaming pass per distinct flip mask instead of the
// reference's copy + apply + axpy per term (ObservablesGPU.hpp:346-362).
#pragma once

#include <algorithm>
#include <functional>
#include <memory>
#include <set>
#include <sstream>
#include <string>
#include <typeinfo>
#include <vector>

#include "StateVectorCudaManaged.hpp"

namespace Pennylane::Algorithms {

template <class T> std::ostream &print_vec(std::ostream &os, const std::vector<T> &v) {
    os << "[";
    for (size_t i = 0; i < v.size(); i++) {
        if (i) os << ", ";
        os << v[i];
    }
    return os << "]";
}

// One Pauli-word view of an observable term: (coefficient, letters, wires).
struct PauliTerm {
    double coeff = 1.0;
    std::string word;
    std::vector<size_t> wires;
};

template <typename T> class ObservableGPU : public std::enable_shared_from_this<ObservableGPU<T>> {
  private:
    [[nodiscard]] virtual bool isEqual(const ObservableGPU<T> &other) const = 0;

  protected:
    ObservableGPU() = default;
    ObservableGPU(const ObservableGPU &) = default;
    ObservableGPU(ObservableGPU &&) noexcept = default;
    ObservableGPU &operator=(const ObservableGPU &) = default;
    ObservableGPU &operator=(ObservableGPU &&) noexcept = default;

  public:
    virtual ~ObservableGPU() = default;
    virtual void applyInPlace(StateVectorCudaManaged<T> &sv) const = 0;
    [[nodiscard]] virtual auto getObsName() const -> std::string = 0;
    [[nodiscard]] virtual auto getWires() const -> std::vector<size_t> = 0;
    // Pauli-word decomposition when the observable is a (sum of) Pauli words.
    [[nodiscard]] virtual bool pauliTerms(std::vector<PauliTerm> &out) const {
        static_cast<void>(out);
        return false;
    }
    [[nodiscard]] bool operator==(const ObservableGPU<T> &other) const {
        return typeid(*this) == typeid(other) && isEqual(other);
    }
    [[nodiscard]] bool operator!=(const ObservableGPU<T> &other) const { return !(*this == other); }
};

template <typename T> class NamedObsGPU final : public ObservableGPU<T> {
  private:
    std::string obs_name_;
    std::vector<size_t> wires_;
    std::vector<T> params_;

    [[nodiscard]] bool isEqual(const ObservableGPU<T> &other) const override {
        const auto &o = static_cast<const NamedObsGPU<T> &>(other);
        return (obs_name_ == o.obs_name_) && (wires_ == o.wires_) && (params_ == o.params_);
    }

  public:
    NamedObsGPU(std::string obs_name, std::vector<size_t> wires, std::vector<T> params = {})
        : obs_name_{std::move(obs_name)}, wires_{std::move(wires)}, params_{std::move(params)} {}

    [[nodiscard]] auto getObsName() const -> std::string override {
        std::ostringstream obs_stream;
        obs_stream << obs_name_;
        print_vec(obs_stream, wires_);
        return obs_stream.str();
    }
    [[nodiscard]] auto getWires() const -> std::vector<size_t> override { return wires_; }
    void applyInPlace(StateVectorCudaManaged<T> &sv) const override {
        sv.applyOperation(obs_name_, wires_, false, params_);
    }
    [[nodiscard]] bool pauliTerms(std::vector<PauliTerm> &out) const override {
        char c = 0;
        if (obs_name_ == "PauliX") c = 'X';
        else if (obs_name_ == "PauliY") c = 'Y';
        else if (obs_name_ == "PauliZ") c = 'Z';
        else if (obs_name_ == "Identity") c = 'I';
        else return false;
        if (wires_.size() != 1) return false;
        out.assign(1, PauliTerm{1.0, std::string(1, c), wires_});
        return true;
    }
};

template <typename T> class HermitianObsGPU final : public ObservableGPU<T> {
  public:
    using MatrixT = std::vector<std::complex<T>>;

  private:
    MatrixT matrix_;
    std::vector<size_t> wires_;

    [[nodiscard]] bool isEqual(const ObservableGPU<T> &other) const override {
        const auto &o = static_cast<const HermitianObsGPU<T> &>(other);
        return (matrix_ == o.matrix_) && (wires_ == o.wires_);
    }

  public:
    HermitianObsGPU(MatrixT matrix, std::vector<size_t> wires) : matrix_{std::move(matrix)}, wires_{std::move(wires)} {
        PL_ABORT_IF(matrix_.size() != (size_t(1) << (2 * wires_.size())), "Hermitian matrix size does not match wires");
    }
    [[nodiscard]] auto getMatrix() const -> const MatrixT { return matrix_; }
    [[nodiscard]] auto getWires() const -> std::vector<size_t> override { return wires_; }
    [[nodiscard]] auto getObsName() const -> std::string override {
        // The name carries a content hash so that different matrices never share a name.
        size_t h = 0;
        for (const auto &v : matrix_) {
            h ^= std::hash<T>{}(v.real()) + 0x9e3779b9 + (h << 6) + (h >> 2);
            h ^= std::hash<T>{}(v.imag()) + 0x9e3779b9 + (h << 6) + (h >> 2);
        }
        std::ostringstream obs_stream;
        obs_stream << "Hermitian" << h;
        return obs_stream.str();
    }
    void applyInPlace(StateVectorCudaManaged<T> &sv) const override {
        std::vector<std::complex<double>> m(matrix_.size());
        for (size_t i = 0; i < m.size(); i++) m[i] = std::complex<double>(matrix_[i].real(), matrix_[i].imag());
        std::vector<int> bits;
        for (size_t w : wires_) {
            PL_ABORT_IF(w >= sv.getNumQubits(), "Wire index out of range");
            bits.push_back(Engine::bit_of(sv.getNumQubits(), w));
        }
        sv.applyMatrixBits(m, bits, {}, {});
    }
};

template <typename T> class TensorProdObsGPU final : public ObservableGPU<T> {
  private:
    std::vector<std::shared_ptr<ObservableGPU<T>>> obs_;
    std::vector<size_t> all_wires_;

    [[nodiscard]] bool isEqual(const ObservableGPU<T> &other) const override {
        const auto &o = static_cast<const TensorProdObsGPU<T> &>(other);
        if (obs_.size() != o.obs_.size()) return false;
        for (size_t i = 0; i < obs_.size(); i++)
            if (*obs_[i] != *o.obs_[i]) return false;
        return true;
    }

  public:
    template <typename... Ts> explicit TensorProdObsGPU(Ts &&...arg) : obs_{std::forward<Ts>(arg)...} {
        std::set<size_t> wires;
        for (const auto &ob : obs_) {
            for (const auto w : ob->getWires()) {
                PL_ABORT_IF(wires.count(w), "All wires in observables must be disjoint.");
                wires.insert(w);
            }
        }
        all_wires_ = std::vector<size_t>(wires.begin(), wires.end());
    }
    static auto create(std::initializer_list<std::shared_ptr<ObservableGPU<T>>> obs)
        -> std::shared_ptr<TensorProdObsGPU<T>> {
        return std::shared_ptr<TensorProdObsGPU<T>>{new TensorProdObsGPU(std::move(obs))};
    }
    static auto create(std::vector<std::shared_ptr<ObservableGPU<T>>> obs) -> std::shared_ptr<TensorProdObsGPU<T>> {
        return std::shared_ptr<TensorProdObsGPU<T>>{new TensorProdObsGPU(std::move(obs))};
    }
    [[nodiscard]] auto getSize() const -> size_t { return obs_.size(); }
    [[nodiscard]] auto getWires() const -> std::vector<size_t> override { return all_wires_; }
    void applyInPlace(StateVectorCudaManaged<T> &sv) const override {
        for (const auto &ob : obs_) ob->applyInPlace(sv);
    }
    [[nodiscard]] auto getObsName() const -> std::string override {
        std::ostringstream s;
        for (size_t i = 0; i < obs_.size(); i++) {
            s << obs_[i]->getObsName();
            if (i + 1 != obs_.size()) s << " @ ";
        }
        return s.str();
    }
    [[nodiscard]] bool pauliTerms(std::vector<PauliTerm> &out) const override {
        PauliTerm t;
        for (const auto &ob : obs_) {
            std::vector<PauliTerm> sub;
            if (!ob->pauliTerms(sub) || sub.size() != 1) return false;
            t.coeff *= sub[0].coeff;
            t.word += sub[0].word;
            t.wires.insert(t.wires.end(), sub[0].wires.begin(), sub[0].wires.end());
        }
        out.assign(1, t);
        return true;
    }
};

template <typename T> class HamiltonianGPU final : public ObservableGPU<T> {
  public:
    using PrecisionT = T;

  private:
    std::vector<T> coeffs_;
    std::vector<std::shared_ptr<ObservableGPU<T>>> obs_;

    [[nodiscard]] bool isEqual(const ObservableGPU<T> &other) const override {
        const auto &o = static_cast<const HamiltonianGPU<T> &>(other);
        if (coeffs_ != o.coeffs_ || obs_.size() != o.obs_.size()) return false;
        for (size_t i = 0; i < obs_.size(); i++)
            if (*obs_[i] != *o.obs_[i]) return false;
        return true;
    }

  public:
    template <typename T1, typename T2>
    HamiltonianGPU(T1 &&arg1, T2 &&arg2) : coeffs_{std::forward<T1>(arg1)}, obs_{std::forward<T2>(arg2)} {
        PL_ASSERT(coeffs_.size() == obs_.size());
    }
    static auto create(std::initializer_list<T> arg1, std::initializer_list<std::shared_ptr<ObservableGPU<T>>> arg2)
        -> std::shared_ptr<HamiltonianGPU<T>> {
        return std::shared_ptr<HamiltonianGPU<T>>(new HamiltonianGPU<T>{std::move(arg1), std::move(arg2)});
    }

    void applyInPlace(StateVectorCudaManaged<T> &sv) const override {
        using CFP_t = typename StateVectorCudaManaged<T>::CFP_t;
        auto buffer = std::make_unique<CUDA::DataBuffer<CFP_t>>(sv.getDataBuffer().getLength(),
                                                                 sv.getDataBuffer().getDevTag());
        std::vector<PauliTerm> terms;
        if (pauliTerms(terms)) {
            std::vector<std::string> words;
            std::vector<std::vector<size_t>> wires;
            std::vector<std::complex<double>> c;
            for (const auto &t : terms) {
                words.push_back(t.word);
                wires.push_back(t.wires);
                c.emplace_back(t.coeff, 0.0);
            }
            sv.applyPauliSumTo(words, wires, c, buffer->getData());
        } else {
            buffer->zeroInit();
            for (size_t term_idx = 0; term_idx < coeffs_.size(); term_idx++) {
                StateVectorCudaManaged<T> tmp(sv);
                obs_[term_idx]->applyInPlace(tmp);
                PL_LGPU_IS_SUCCESS(lgpu_axpy(double(coeffs_[term_idx]), 0.0, tmp.getData(), buffer->getData(),
                                             uint32_t(sv.getNumQubits()), StateVectorCudaManaged<T>::dt(),
                                             sv.lstream()));
                tmp.sync();
            }
        }
        sv.updateData(std::move(buffer));
    }

    [[nodiscard]] bool pauliTerms(std::vector<PauliTerm> &out) const override {
        out.clear();
        for (size_t i = 0; i < obs_.size(); i++) {
            std::vector<PauliTerm> sub;
            if (!obs_[i]->pauliTerms(sub)) return false;
            for (auto &t : sub) {
                t.coeff *= double(coeffs_[i]);
                out.push_back(t);
            }
        }
        return true;
    }

    [[nodiscard]] auto getWires() const -> std::vector<size_t> override {
        std::set<size_t> wires;
        for (const auto &ob : obs_)
            for (auto w : ob->getWires()) wires.insert(w);
        return std::vector<size_t>(wires.begin(), wires.end());
    }
    [[nodiscard]] auto getObsName() const -> std::string override {
        std::ostringstream ss;
        ss << "Hamiltonian: { 'coeffs' : ";
        print_vec(ss, coeffs_);
        ss << ", 'observables' : [";
        for (size_t t = 0; t < coeffs_.size(); t++) {
            ss << obs_[t]->getObsName();
            if (t + 1 != coeffs_.size()) ss << ", ";
        }
        ss << "]}";
        return ss.str();
    }
    [[nodiscard]] auto getCoeffs() const -> const std::vector<T> & { return coeffs_; }
    [[nodiscard]] auto getObs() const -> const std::vector<std::shared_ptr<ObservableGPU<T>>> & { return obs_; }
};

template <typename T> class SparseHamiltonianGPU final : public ObservableGPU<T> {
  public:
    using PrecisionT = T;
    using IdxT = typename std::conditional<std::is_same<T, float>::value, int32_t, int64_t>::type;

  private:
    std::vector<std::complex<T>> data_;
    std::vector<IdxT> indices_;
    std::vector<IdxT> offsets_;
    std::vector<std::size_t> wires_;

    [[nodiscard]] bool isEqual(const ObservableGPU<T> &other) const override {
        const auto &o = static_cast<const SparseHamiltonianGPU<T> &>(other);
        return data_ == o.data_ && indices_ == o.indices_ && offsets_ == o.offsets_;
    }

  public:
    template <typename T1, typename T2, typename T3 = T2, typename T4 = std::vector<std::size_t>>
    SparseHamiltonianGPU(T1 &&arg1, T2 &&arg2, T3 &&arg3, T4 &&arg4)
        : data_{std::forward<T1>(arg1)}, indices_{std::forward<T2>(arg2)}, offsets_{std::forward<T3>(arg3)},
          wires_{std::forward<T4>(arg4)} {
        PL_ASSERT(data_.size() == indices_.size());
    }
    static auto create(std::initializer_list<std::complex<T>> arg1, std::initializer_list<IdxT> arg2,
                       std::initializer_list<IdxT> arg3, std::initializer_list<std::size_t> arg4)
        -> std::shared_ptr<SparseHamiltonianGPU<T>> {
        return std::shared_ptr<SparseHamiltonianGPU<T>>(
            new SparseHamiltonianGPU<T>{std::move(arg1), std::move(arg2), std::move(arg3), std::move(arg4)});
    }

    void applyInPlace(StateVectorCudaManaged<T> &sv) const override {
        PL_ABORT_IF_NOT(wires_.size() == sv.getNumQubits(), "SparseH wire count does not match state-vector size");
        using CFP_t = typename StateVectorCudaManaged<T>::CFP_t;
        auto sp = sv.uploadCSR(offsets_.data(), offsets_.size(), indices_.data(), data_.data(), data_.size());
        auto out = std::make_unique<CUDA::DataBuffer<CFP_t>>(sv.getDataBuffer().getLength(),
                                                             sv.getDataBuffer().getDevTag());
        PL_LGPU_IS_SUCCESS(lgpu_spmv_csr(sp.off->getData(), sp.col->getData(), sp.val->getData(), sv.getData(),
                                         out->getData(), uint32_t(sv.getNumQubits()), StateVectorCudaManaged<T>::dt(),
                                         sv.lstream()));
        sv.sync();
        sv.updateData(std::move(out));
    }
    [[nodiscard]] auto getObsName() const -> std::string override {
        std::ostringstream ss;
        ss << "SparseHamiltonian: {\n'data' : ";
        for (const auto &d : data_) ss << d;
        ss << ",\n'indices' : ";
        for (const auto &d : indices_) ss << d;
        ss << ",\n'offsets' : ";
        for (const auto &d : offsets_) ss << d;
        ss << "\n}";
        return ss.str();
    }
    [[nodiscard]] auto getWires() const -> std::vector<size_t> override { return wires_; }
};

} // namespace Pennylane::Algorithms
