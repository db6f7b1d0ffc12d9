// StateVectorCudaManaged<Precision>: the drop-in device state vector.
//
// Same public interface as the reference
// (src/simulator/StateVectorCudaManaged.hpp:69-1714): constructors, basis /
// sparse state preparation, the applyOperation dispatcher and its batched
// overloads, every apply<Gate> method, the applyGenerator* methods, the three
// expval overloads, sparse and Pauli-word expectations, probability and
// generate_samples.  Every computation is a call into the sm_103a kernels of
// liblgpu_gb300 through the C ABI in lgpu.h; there is no cuStateVec, cuBLAS
// or cuSPARSE underneath.
#pragma once

#include <algorithm>
#include <complex>
#include <cstdint>
#include <functional>
#include <map>
#include <memory>
#include <numeric>
#include <optional>
#include <random>
#include <string>
#include <unordered_map>
#include <vector>

#include "GateLowering.hpp"
#include "StateVectorCudaBase.hpp"

namespace Pennylane {

template <class Precision>
class StateVectorCudaManaged : public StateVectorCudaBase<Precision, StateVectorCudaManaged<Precision>> {
  private:
    using BaseType = StateVectorCudaBase<Precision, StateVectorCudaManaged>;
    using cd = std::complex<double>;

  public:
    using PrecisionT = Precision;
    using ComplexT = std::complex<PrecisionT>;
    using CFP_t = typename BaseType::CFP_t;
    using GateType = CFP_t *;

    StateVectorCudaManaged() = delete;
    StateVectorCudaManaged(size_t num_qubits)
        : BaseType(num_qubits), handle_(CUDA::make_shared_cusv_handle()),
          ctx_(std::make_shared<CUDA::LgpuContext>(0)) {
        BaseType::initSV();
    }

    StateVectorCudaManaged(size_t num_qubits, const CUDA::DevTag<int> &dev_tag, bool alloc = true,
                           CUDA::SharedCusvHandle cusvhandle_in = CUDA::make_shared_cusv_handle(),
                           CUDA::SharedCublasCaller cublascaller_in = CUDA::make_shared_cublas_caller(),
                           CUDA::SharedCusparseHandle cusparsehandle_in = CUDA::make_shared_cusparse_handle())
        : BaseType(num_qubits, dev_tag, alloc), handle_(std::move(cusvhandle_in)),
          ctx_(std::make_shared<CUDA::LgpuContext>(dev_tag.getDeviceID())) {
        static_cast<void>(cublascaller_in);
        static_cast<void>(cusparsehandle_in);
        if (alloc) BaseType::initSV();
    }

    StateVectorCudaManaged(const CFP_t *gpu_data, size_t length) : StateVectorCudaManaged(Util::log2(length)) {
        BaseType::CopyGpuDataToGpuIn(gpu_data, length, false);
    }

    StateVectorCudaManaged(const CFP_t *gpu_data, size_t length, CUDA::DevTag<int> dev_tag,
                           CUDA::SharedCusvHandle handle_in = CUDA::make_shared_cusv_handle(),
                           CUDA::SharedCublasCaller cublascaller_in = CUDA::make_shared_cublas_caller(),
                           CUDA::SharedCusparseHandle cusparsehandle_in = CUDA::make_shared_cusparse_handle())
        : StateVectorCudaManaged(Util::log2(length), dev_tag, true, std::move(handle_in), std::move(cublascaller_in),
                                 std::move(cusparsehandle_in)) {
        BaseType::CopyGpuDataToGpuIn(gpu_data, length, false);
    }

    StateVectorCudaManaged(const std::complex<Precision> *host_data, size_t length)
        : StateVectorCudaManaged(Util::log2(length)) {
        PL_ABORT_IF_NOT(Util::exp2(Util::log2(length)) == length, "State length must be a power of two");
        BaseType::CopyHostDataToGpu(host_data, length, false);
    }

    StateVectorCudaManaged(const StateVectorCudaManaged &other)
        : BaseType(other.getNumQubits(), other.getDataBuffer().getDevTag()), handle_(other.handle_),
          ctx_(std::make_shared<CUDA::LgpuContext>(other.getDataBuffer().getDevTag().getDeviceID())),
          seed_(other.seed_) {
        BaseType::CopyGpuDataToGpuIn(other);
    }

    // Work queued on this state's stream may still use its scratch context,
    // which goes back to the library's free list with it.
    ~StateVectorCudaManaged() { lgpu_stream_sync(BaseType::lstream()); }

    // ---- state preparation -------------------------------------------------
    void setBasisState(const std::complex<Precision> &value, const size_t index, const bool async = false) {
        PL_ABORT_IF(index >= BaseType::getLength(), "Basis-state index out of range");
        PL_LGPU_IS_SUCCESS(lgpu_set_basis(BaseType::getData(), nq(), dt(), index, double(value.real()),
                                          double(value.imag()), BaseType::lstream()));
        if (!async) sync();
    }

    template <class index_type, size_t thread_per_block = 256>
    void setStateVector(const index_type num_indices, const std::complex<Precision> *values,
                        const index_type *indices, const bool async = false) {
        const size_t cnt = static_cast<size_t>(num_indices);
        std::vector<int64_t> idx(cnt);
        for (size_t i = 0; i < cnt; i++) {
            PL_ABORT_IF(indices[i] < 0 || static_cast<size_t>(indices[i]) >= BaseType::getLength(),
                        "setStateVector: index out of range");
            idx[i] = static_cast<int64_t>(indices[i]);
        }
        const auto dev = BaseType::getDataBuffer().getDevTag().getDeviceID();
        const auto stream = BaseType::getDataBuffer().getDevTag().getStreamID();
        CUDA::DataBuffer<int64_t, int> d_idx{cnt, dev, stream, true};
        CUDA::DataBuffer<CFP_t, int> d_val{cnt, dev, stream, true};
        if (cnt) {
            d_idx.CopyHostDataToGpu(idx.data(), cnt, async);
            d_val.CopyHostDataToGpu(reinterpret_cast<const CFP_t *>(values), cnt, async);
        }
        PL_LGPU_IS_SUCCESS(lgpu_scatter(BaseType::getData(), nq(), dt(), d_val.getData(), d_idx.getData(), cnt, 1,
                                        BaseType::lstream()));
        sync();  // the temporary index/value buffers die here
    }

    // ---- dispatcher -----------------------------------------------------------
    void applyOperation(const std::string &opName, const std::vector<size_t> &wires, bool adjoint = false,
                        const std::vector<Precision> &params = {0.0}, const std::vector<CFP_t> &gate_matrix = {}) {
        std::vector<cd> um = Engine::to_cd(gate_matrix);
        const std::vector<double> p(params.begin(), params.end());
        if (um.empty() && !known_gate(opName)) {
            // The reference caches user matrices by (name, param[0]) and reuses
            // them for later calls without a matrix (cuGateCache.hpp:197-228).
            auto it = user_gate_cache_.find(key(opName, p));
            PL_ABORT_IF(it == user_gate_cache_.end(), ("Currently unsupported gate: " + opName).c_str());
            um = it->second;
        } else if (!um.empty() && !known_gate(opName)) {
            user_gate_cache_[key(opName, p)] = um;
        }
        applyDesc(Engine::lower_operation(nq(), opName, wires, adjoint, p, um));
    }

    void applyOperation_std(const std::string &opName, const std::vector<size_t> &wires, bool adjoint = false,
                            const std::vector<Precision> &params = {0.0},
                            const std::vector<std::complex<Precision>> &gate_matrix = {}) {
        std::vector<CFP_t> m(gate_matrix.size());
        for (size_t i = 0; i < m.size(); i++) m[i] = cuUtil::complexToCu<std::complex<Precision>>(gate_matrix[i]);
        applyOperation(opName, wires, adjoint, params, m);
    }

    // Multi-op variants.  Consecutive ops are lowered, planned into
    // shared-memory fused blocks and applied with one HBM pass per block.
    void applyOperation(const std::vector<std::string> &opNames, const std::vector<std::vector<size_t>> &wires,
                        const std::vector<bool> &adjoints, const std::vector<std::vector<Precision>> &params) {
        PL_ABORT_IF(opNames.size() != wires.size(), "Incompatible number of ops and wires");
        PL_ABORT_IF(opNames.size() != adjoints.size(), "Incompatible number of ops and adjoints");
        PL_ABORT_IF(opNames.size() != params.size(), "Incompatible number of ops and params");
        std::vector<Engine::GateDesc> descs;
        descs.reserve(opNames.size());
        for (size_t i = 0; i < opNames.size(); i++) {
            const std::vector<double> p(params[i].begin(), params[i].end());
            std::vector<cd> um;
            if (!known_gate(opNames[i])) {
                auto it = user_gate_cache_.find(key(opNames[i], p));
                PL_ABORT_IF(it == user_gate_cache_.end(), ("Currently unsupported gate: " + opNames[i]).c_str());
                um = it->second;
            }
            descs.push_back(Engine::lower_operation(nq(), opNames[i], wires[i], adjoints[i], p, um));
        }
        applyDescs(descs);
    }

    void applyOperation(const std::vector<std::string> &opNames, const std::vector<std::vector<size_t>> &wires,
                        const std::vector<bool> &adjoints) {
        PL_ABORT_IF(opNames.size() != wires.size(), "Incompatible number of ops and wires");
        PL_ABORT_IF(opNames.size() != adjoints.size(), "Incompatible number of ops and adjoints");
        std::vector<std::vector<Precision>> params(opNames.size(), std::vector<Precision>{0.0});
        applyOperation(opNames, wires, adjoints, params);
    }

    // ---- per-gate methods (StateVectorCudaManaged.hpp:320-560) -----------------
    // Non-parametric gates: wires[:-1] are controls, wires.back() the target.
    inline void applyIdentity(const std::vector<size_t> &wires, bool adjoint) {
        static_cast<void>(wires);
        static_cast<void>(adjoint);
    }
    inline void applyPauliX(const std::vector<size_t> &wires, bool adjoint) { ctrl_last("PauliX", wires, adjoint); }
    inline void applyPauliY(const std::vector<size_t> &wires, bool adjoint) { ctrl_last("PauliY", wires, adjoint); }
    inline void applyPauliZ(const std::vector<size_t> &wires, bool adjoint) { ctrl_last("PauliZ", wires, adjoint); }
    inline void applyHadamard(const std::vector<size_t> &wires, bool adjoint) { ctrl_last("Hadamard", wires, adjoint); }
    inline void applyS(const std::vector<size_t> &wires, bool adjoint) { ctrl_last("S", wires, adjoint); }
    inline void applyT(const std::vector<size_t> &wires, bool adjoint) { ctrl_last("T", wires, adjoint); }
    inline void applyCNOT(const std::vector<size_t> &wires, bool adjoint) { ctrl_last("PauliX", wires, adjoint); }
    inline void applyCY(const std::vector<size_t> &wires, bool adjoint) { ctrl_last("PauliY", wires, adjoint); }
    inline void applyCZ(const std::vector<size_t> &wires, bool adjoint) { ctrl_last("PauliZ", wires, adjoint); }
    inline void applyToffoli(const std::vector<size_t> &wires, bool adjoint) { ctrl_last("PauliX", wires, adjoint); }
    inline void applySWAP(const std::vector<size_t> &wires, bool adjoint) {
        applyOperation("SWAP", wires, adjoint);
    }
    inline void applyCSWAP(const std::vector<size_t> &wires, bool adjoint) { applyOperation("CSWAP", wires, adjoint); }

    // Rotations: wires[:-1] are controls (StateVectorCudaManaged.hpp:370-386).
    inline void applyRX(const std::vector<size_t> &wires, bool adjoint, Precision param) {
        rot_last("RX", wires, adjoint, param);
    }
    inline void applyRY(const std::vector<size_t> &wires, bool adjoint, Precision param) {
        rot_last("RY", wires, adjoint, param);
    }
    inline void applyRZ(const std::vector<size_t> &wires, bool adjoint, Precision param) {
        rot_last("RZ", wires, adjoint, param);
    }
    inline void applyCRX(const std::vector<size_t> &wires, bool adjoint, Precision param) { applyRX(wires, adjoint, param); }
    inline void applyCRY(const std::vector<size_t> &wires, bool adjoint, Precision param) { applyRY(wires, adjoint, param); }
    inline void applyCRZ(const std::vector<size_t> &wires, bool adjoint, Precision param) { applyRZ(wires, adjoint, param); }
    inline void applyRot(const std::vector<size_t> &wires, bool adjoint, Precision p0, Precision p1, Precision p2) {
        applyOperation("Rot", wires, adjoint, {p0, p1, p2});
    }
    inline void applyRot(const std::vector<size_t> &wires, bool adjoint, const std::vector<Precision> &params) {
        applyRot(wires, adjoint, params[0], params[1], params[2]);
    }
    inline void applyCRot(const std::vector<size_t> &wires, bool adjoint, Precision p0, Precision p1, Precision p2) {
        applyOperation("CRot", wires, adjoint, {p0, p1, p2});
    }
    inline void applyCRot(const std::vector<size_t> &wires, bool adjoint, const std::vector<Precision> &params) {
        applyCRot(wires, adjoint, params[0], params[1], params[2]);
    }
    inline void applyPhaseShift(const std::vector<size_t> &wires, bool adjoint, Precision param) {
        applyOperation("PhaseShift", wires, adjoint, {param});
    }
    inline void applyControlledPhaseShift(const std::vector<size_t> &wires, bool adjoint, Precision param) {
        applyOperation("PhaseShift", wires, adjoint, {param});
    }
    inline void applyIsingXX(const std::vector<size_t> &wires, bool adjoint, Precision param) {
        applyOperation("IsingXX", wires, adjoint, {param});
    }
    inline void applyIsingYY(const std::vector<size_t> &wires, bool adjoint, Precision param) {
        applyOperation("IsingYY", wires, adjoint, {param});
    }
    inline void applyIsingZZ(const std::vector<size_t> &wires, bool adjoint, Precision param) {
        applyOperation("IsingZZ", wires, adjoint, {param});
    }
    inline void applyMultiRZ(const std::vector<size_t> &wires, bool adjoint, Precision param) {
        applyOperation("MultiRZ", wires, adjoint, {param});
    }
    inline void applySingleExcitation(const std::vector<size_t> &wires, bool adjoint, Precision param) {
        applyOperation("SingleExcitation", wires, adjoint, {param});
    }
    inline void applySingleExcitationMinus(const std::vector<size_t> &wires, bool adjoint, Precision param) {
        applyOperation("SingleExcitationMinus", wires, adjoint, {param});
    }
    inline void applySingleExcitationPlus(const std::vector<size_t> &wires, bool adjoint, Precision param) {
        applyOperation("SingleExcitationPlus", wires, adjoint, {param});
    }
    inline void applyDoubleExcitation(const std::vector<size_t> &wires, bool adjoint, Precision param) {
        applyOperation("DoubleExcitation", wires, adjoint, {param});
    }
    inline void applyDoubleExcitationMinus(const std::vector<size_t> &wires, bool adjoint, Precision param) {
        applyOperation("DoubleExcitationMinus", wires, adjoint, {param});
    }
    inline void applyDoubleExcitationPlus(const std::vector<size_t> &wires, bool adjoint, Precision param) {
        applyOperation("DoubleExcitationPlus", wires, adjoint, {param});
    }

    // ---- generators (StateVectorCudaManaged.hpp:563-688) ------------------------
    inline void applyGeneratorIsingXX(const std::vector<size_t> &wires, bool adjoint) { gen("IsingXX", wires, adjoint); }
    inline void applyGeneratorIsingYY(const std::vector<size_t> &wires, bool adjoint) { gen("IsingYY", wires, adjoint); }
    inline void applyGeneratorIsingZZ(const std::vector<size_t> &wires, bool adjoint) { gen("IsingZZ", wires, adjoint); }
    inline void applyGeneratorSingleExcitation(const std::vector<size_t> &wires, bool adjoint) {
        gen("SingleExcitation", wires, adjoint);
    }
    inline void applyGeneratorSingleExcitationMinus(const std::vector<size_t> &wires, bool adjoint) {
        gen("SingleExcitationMinus", wires, adjoint);
    }
    inline void applyGeneratorSingleExcitationPlus(const std::vector<size_t> &wires, bool adjoint) {
        gen("SingleExcitationPlus", wires, adjoint);
    }
    inline void applyGeneratorDoubleExcitation(const std::vector<size_t> &wires, bool adjoint) {
        gen("DoubleExcitation", wires, adjoint);
    }
    inline void applyGeneratorDoubleExcitationMinus(const std::vector<size_t> &wires, bool adjoint) {
        gen("DoubleExcitationMinus", wires, adjoint);
    }
    inline void applyGeneratorDoubleExcitationPlus(const std::vector<size_t> &wires, bool adjoint) {
        gen("DoubleExcitationPlus", wires, adjoint);
    }
    inline void applyGeneratorMultiRZ(const std::vector<size_t> &wires, bool adjoint) {
        for (size_t w : wires) applyPauliZ({w}, adjoint);
    }

    // Generator of `opName` applied on `wires` (GateGenerators.hpp); returns
    // the scale factor of the reference's scaling_factors map.  The
    // generator acts on the op's wires in order (controls first).
    double applyGeneratorOf(const std::string &opName, const std::vector<size_t> &wires, bool adjoint) {
        std::vector<int> bits;
        for (size_t w : wires) {
            PL_ABORT_IF(w >= nq(), "Wire index out of range");
            bits.push_back(Engine::bit_of(nq(), w));
        }
        std::vector<cd> g;
        double scale = 0;
        PL_ABORT_IF_NOT(Engine::generator_of(opName, bits.size(), g, scale), "No generator for the operation");
        if (adjoint) g = Engine::dagger(g);
        if (opName == "MultiRZ") {
            for (int b : bits) applyMatrixBits({1.0, 0.0, 0.0, -1.0}, {b}, {}, {});
        } else {
            applyMatrixBits(g, bits, {}, {});
        }
        return scale;
    }

    // ---- expectation values (StateVectorCudaManaged.hpp:702-780) ----------------
    auto expval(const std::string &obsName, const std::vector<size_t> &wires,
                const std::vector<Precision> &params = {0.0}, const std::vector<CFP_t> &gate_matrix = {}) -> CFP_t {
        std::vector<cd> m = Engine::to_cd(gate_matrix);
        if (m.empty()) {
            const std::vector<double> p(params.begin(), params.end());
            auto it = user_gate_cache_.find(key(obsName, p));
            if (it != user_gate_cache_.end()) {
                m = it->second;
            } else if (!Engine::constant_gate(obsName, m)) {
                throw LightningException("Currently unsupported observable: " + obsName);
            }
        }
        return expvalMatrixWires(m, wires);
    }
    auto expval(const std::string &obsName, const std::vector<size_t> &wires,
                const std::vector<Precision> &params = {0.0},
                const std::vector<std::complex<Precision>> &gate_matrix = {}) -> CFP_t {
        std::vector<CFP_t> m(gate_matrix.size());
        for (size_t i = 0; i < m.size(); i++) m[i] = cuUtil::complexToCu<std::complex<Precision>>(gate_matrix[i]);
        return expval(obsName, wires, params, m);
    }
    auto expval(const std::vector<size_t> &wires, const std::vector<std::complex<Precision>> &gate_matrix) -> CFP_t {
        PL_ABORT_IF(gate_matrix.empty(), "Currently unsupported observable");
        std::vector<cd> m(gate_matrix.size());
        for (size_t i = 0; i < m.size(); i++) m[i] = cd(gate_matrix[i].real(), gate_matrix[i].imag());
        return expvalMatrixWires(m, wires);
    }

    // <psi|M|psi> for a dense PennyLane-ordered matrix on wires.
    auto expvalMatrixWires(const std::vector<cd> &m, const std::vector<size_t> &wires) -> CFP_t {
        const size_t t = wires.size();
        PL_ABORT_IF(m.size() != (size_t(1) << (2 * t)), "Matrix size does not match the number of wires");
        std::vector<int32_t> bits(t);
        for (size_t k = 0; k < t; k++) {
            PL_ABORT_IF(wires[k] >= nq(), "Wire index out of range");
            bits[k] = Engine::bit_of(nq(), wires[k]);
        }
        double out[2] = {0, 0};
        PL_LGPU_IS_SUCCESS(lgpu_expval_matrix(ctx(), BaseType::getData(), nq(), dt(),
                                              reinterpret_cast<const double *>(m.data()), uint32_t(t), bits.data(),
                                              out, 0, BaseType::lstream()));
        return CFP_t{static_cast<Precision>(out[0]), static_cast<Precision>(out[1])};
    }

    // <psi|H|psi> for a CSR matrix (StateVectorCudaManaged.hpp:795-922).
    template <class index_type>
    auto getExpectationValueOnSparseSpMV(const index_type *csrOffsets_ptr, const index_type csrOffsets_size,
                                         const index_type *columns_ptr, const std::complex<Precision> *values_ptr,
                                         const index_type numNNZ) -> Precision {
        const size_t nrows = static_cast<size_t>(csrOffsets_size) - 1;
        PL_ABORT_IF(nrows != BaseType::getLength(), "Sparse matrix dimension does not match the state vector");
        SparseDev sp = uploadCSR(csrOffsets_ptr, size_t(csrOffsets_size), columns_ptr, values_ptr, size_t(numNNZ));
        double out[2] = {0, 0};
        PL_LGPU_IS_SUCCESS(lgpu_expval_csr(ctx(), sp.off->getData(), sp.col->getData(), sp.val->getData(),
                                           BaseType::getData(), nq(), dt(), out, 0, BaseType::lstream()));
        return static_cast<Precision>(out[0]);
    }

    // ---- probabilities (StateVectorCudaManaged.hpp:931-970) ---------------------
    // Output bit k corresponds to wires[k] ("column-major" order).
    auto probability(const std::vector<size_t> &wires) -> std::vector<double> {
        std::vector<int32_t> bits(wires.size());
        for (size_t k = 0; k < wires.size(); k++) {
            PL_ABORT_IF(wires[k] >= nq(), "Wire index out of range");
            bits[k] = Engine::bit_of(nq(), wires[k]);
        }
        std::vector<double> probs(size_t(1) << wires.size());
        if (wires.empty()) {
            probs[0] = 1.0;
            return probs;
        }
        PL_LGPU_IS_SUCCESS(lgpu_probs(ctx(), BaseType::getData(), nq(), dt(), uint32_t(wires.size()), bits.data(),
                                      probs.data(), 0, BaseType::lstream()));
        return probs;
    }

    // ---- sampling (StateVectorCudaManaged.hpp:982-1061) -------------------------
    // Draws: std::mt19937 + uniform_real_distribution<Precision>(0, 1), seeded
    // from std::random_device unless setSeed() fixed the seed.  Samples come
    // back in ascending index order, decoded to (shots x n) bits, wire 0 first.
    auto generate_samples(size_t num_samples) -> std::vector<size_t> {
        const auto idx = generate_sample_indices(num_samples, true);
        const size_t n = nq();
        std::vector<size_t> samples(num_samples * n, 0);
        for (size_t i = 0; i < num_samples; i++)
            for (size_t j = 0; j < n; j++) samples[i * n + (n - 1 - j)] = (idx[i] >> j) & 1U;
        return samples;
    }

    auto generate_sample_indices(size_t num_samples, bool sorted) -> std::vector<uint64_t> {
        std::vector<double> draws(num_samples);
        std::mt19937 gen(seed_ ? static_cast<std::mt19937::result_type>(*seed_) : std::random_device{}());
        std::uniform_real_distribution<Precision> dis(0.0, 1.0);
        for (size_t i = 0; i < num_samples; i++) {
            Precision r = dis(gen);
            if (!(r < Precision(1))) r = std::nextafter(Precision(1), Precision(0));
            draws[i] = double(r);
        }
        if (seed_) seed_ = *seed_ + 1;  // next call continues with a new stream
        std::vector<uint64_t> idx(num_samples);
        if (num_samples)
            PL_LGPU_IS_SUCCESS(lgpu_sample(ctx(), BaseType::getData(), nq(), dt(), draws.data(), num_samples,
                                           idx.data(), BaseType::lstream()));
        if (sorted) std::sort(idx.begin(), idx.end());
        return idx;
    }

    void setSeed(uint64_t seed) { seed_ = seed; }
    void clearSeed() { seed_.reset(); }

    // ---- Pauli words (StateVectorCudaManaged.hpp:1071-1148) ---------------------
    auto getExpectationValuePauliWords(const std::vector<std::string> &pauli_words,
                                       const std::vector<std::vector<size_t>> &tgts,
                                       const std::complex<Precision> *coeffs) -> Precision {
        PL_ABORT_IF(pauli_words.size() != tgts.size(), "Number of Pauli words and wire lists differ");
        std::vector<uint64_t> flip, sgn;
        std::vector<uint8_t> ny;
        pauliMasks(pauli_words, tgts, flip, sgn, ny);
        std::vector<double> ev(pauli_words.size(), 0.0);
        if (!ev.empty())
            PL_LGPU_IS_SUCCESS(lgpu_expval_pauli_words(ctx(), BaseType::getData(), nq(), dt(), uint32_t(ev.size()),
                                                       flip.data(), sgn.data(), ny.data(), ev.data(), 0,
                                                       BaseType::lstream()));
        // FP64 coefficient sum for both precisions.
        std::complex<double> result{0, 0};
        for (size_t i = 0; i < ev.size(); i++)
            result += ev[i] * std::complex<double>(double(coeffs[i].real()), double(coeffs[i].imag()));
        return static_cast<Precision>(result.real());
    }

    void pauliMasks(const std::vector<std::string> &words, const std::vector<std::vector<size_t>> &tgts,
                    std::vector<uint64_t> &flip, std::vector<uint64_t> &sgn, std::vector<uint8_t> &ny) const {
        flip.assign(words.size(), 0);
        sgn.assign(words.size(), 0);
        ny.assign(words.size(), 0);
        for (size_t t = 0; t < words.size(); t++) {
            PL_ABORT_IF(words[t].size() != tgts[t].size(), "Pauli word and wire list lengths differ");
            for (size_t k = 0; k < words[t].size(); k++) {
                PL_ABORT_IF(tgts[t][k] >= nq(), "Wire index out of range");
                const uint64_t b = uint64_t(1) << Engine::bit_of(nq(), tgts[t][k]);
                PL_ABORT_IF(((flip[t] | sgn[t]) & b) != 0 && words[t][k] != 'I', "Repeated wire in a Pauli word");
                switch (words[t][k]) {
                case 'X': flip[t] |= b; break;
                case 'Y': flip[t] |= b; sgn[t] |= b; ny[t]++; break;
                case 'Z': sgn[t] |= b; break;
                case 'I': break;
                default: PL_ABORT("Invalid character in Pauli word");
                }
            }
        }
    }

    // out = sum_t c_t P_t |this>  (one pass per distinct flip mask)
    void applyPauliSumTo(const std::vector<std::string> &words, const std::vector<std::vector<size_t>> &tgts,
                         const std::vector<std::complex<double>> &coeffs, CFP_t *out) const {
        std::vector<uint64_t> flip, sgn;
        std::vector<uint8_t> ny;
        pauliMasks(words, tgts, flip, sgn, ny);
        PL_LGPU_IS_SUCCESS(lgpu_apply_pauli_sum(BaseType::getData(), out, nq(), dt(), uint32_t(words.size()),
                                                reinterpret_cast<const double *>(coeffs.data()), flip.data(),
                                                sgn.data(), ny.data(), BaseType::lstream()));
    }

    // ---- engine-level helpers ---------------------------------------------------
    // Dense matrix (PennyLane order, already in final form) on state bits.
    void applyMatrixBits(const std::vector<cd> &m, const std::vector<int> &tgts, const std::vector<int> &ctrls,
                         const std::vector<int> &cvals) {
        std::vector<int32_t> t(tgts.begin(), tgts.end()), c(ctrls.begin(), ctrls.end()), v(cvals.begin(), cvals.end());
        if (v.empty()) v.assign(c.size(), 1);
        PL_LGPU_IS_SUCCESS(lgpu_apply_matrix(BaseType::getData(), nq(), dt(), reinterpret_cast<const double *>(m.data()),
                                             uint32_t(t.size()), t.data(), uint32_t(c.size()), c.data(), v.data(), 0,
                                             BaseType::lstream()));
    }

    // The same lowered gate on several states of this size in one launch per
    // gate (the states share this state's stream).
    void applyDescMulti(const Engine::GateDesc &d, const std::vector<void *> &states) const {
        if (states.empty() || d.kind == Engine::GateDesc::IDENTITY) return;
        std::vector<int32_t> t(d.tgts.begin(), d.tgts.end()), c(d.ctrls.begin(), d.ctrls.end()),
            v(d.cvals.begin(), d.cvals.end());
        if (v.empty()) v.assign(c.size(), 1);
        if (d.kind == Engine::GateDesc::MATRIX) {
            PL_LGPU_IS_SUCCESS(lgpu_apply_matrix_multi(states.data(), uint32_t(states.size()), nq(), dt(),
                                                       reinterpret_cast<const double *>(d.matrix.data()),
                                                       uint32_t(t.size()), t.data(), uint32_t(c.size()), c.data(),
                                                       v.data(), 0, BaseType::lstream()));
        } else {
            PL_LGPU_IS_SUCCESS(lgpu_apply_pauli_rotation_multi(states.data(), uint32_t(states.size()), nq(), dt(),
                                                               d.angle, uint32_t(t.size()), t.data(),
                                                               d.paulis.c_str(), uint32_t(c.size()), c.data(),
                                                               v.data(), BaseType::lstream()));
        }
    }

    void applyDesc(const Engine::GateDesc &d) {
        switch (d.kind) {
        case Engine::GateDesc::IDENTITY: return;
        case Engine::GateDesc::MATRIX: applyMatrixBits(d.matrix, d.tgts, d.ctrls, d.cvals); return;
        case Engine::GateDesc::PAULI_ROT: {
            std::vector<int32_t> t(d.tgts.begin(), d.tgts.end()), c(d.ctrls.begin(), d.ctrls.end()),
                v(d.cvals.begin(), d.cvals.end());
            PL_LGPU_IS_SUCCESS(lgpu_apply_pauli_rotation(BaseType::getData(), nq(), dt(), d.angle, uint32_t(t.size()),
                                                         t.data(), d.paulis.c_str(), uint32_t(c.size()), c.data(),
                                                         v.data(), BaseType::lstream()));
            return;
        }
        }
    }

    // Fusion is on by default for multi-op calls; setFusion(false) applies
    // the ops one kernel each (the plain per-gate path).
    // tile_bits / min_low_bits (0 = default) set the planner's tile size and
    // the shortest contiguous low run of a tile.
    void setFusion(bool on, int tile_bits = 0, int min_low_bits = 0) {
        fusion_ = on;
        if (tile_bits > 0) fusion_tile_bits_ = tile_bits;
        if (min_low_bits > 0) fusion_min_low_bits_ = min_low_bits;
    }
    [[nodiscard]] bool getFusion() const { return fusion_; }
    [[nodiscard]] int fusionTileBits() const {
        if (fusion_tile_bits_ > 0) return fusion_tile_bits_;
        return 12;  // 32 KB (complex64, double-buffered) / 64 KB (complex128) tiles: three CTAs per SM
    }
    // Tile bits above the contiguous low run (lgpu_apply_fused_block takes up
    // to 8).
    static constexpr int kFusionMaxHighBits = 8;
    // Shortest contiguous low run of a tile: 2^5 amplitudes keep every
    // segment at least 256 bytes long.
    [[nodiscard]] int fusionMinLowBits() const {
        if (fusion_min_low_bits_ > 0) return fusion_min_low_bits_;
        return 5;
    }

    void applyDescs(std::vector<Engine::GateDesc> descs) {
        if (!fusion_ || descs.size() < 2) {
            for (const auto &d : descs) applyDesc(d);
            return;
        }
        // 1- and 2-target Pauli rotations become matrices so they can be fused.
        for (auto &d : descs) {
            if (d.kind == Engine::GateDesc::PAULI_ROT && d.tgts.size() <= 2 && d.ctrls.empty()) {
                std::vector<int> bits;
                std::vector<cd> m;
                if (Engine::dense_on_bits(d, bits, m, 2)) {
                    d.kind = Engine::GateDesc::MATRIX;
                    d.matrix = m;
                }
            }
        }
        Engine::merge_1q_runs(descs);
        const int kmax = std::min<int>(fusionTileBits(), int(nq()));
        const auto plan = Engine::plan_fusion(descs, nq(), kmax, std::min<int>(fusionMinLowBits(), kmax), 2,
                                              size_t(kFusionMaxHighBits));
        // complex128: consecutive fused blocks pass the state on in float-float
        // form (lgpu_apply_fused_block_ff); the last block of such a run
        // converts it back
        const bool ff_ok = dt() == LGPU_C128;
        bool in_ff = false;
        for (size_t bi = 0; bi < plan.size(); bi++) {
            const auto &blk = plan[bi];
            if (blk.tile_bits.empty()) {
                for (size_t gi : blk.gates) applyDesc(descs[gi]);
                continue;
            }
            std::vector<lgpu_fused_gate_t> fg;
            for (size_t gi : blk.gates) {
                const auto &d = descs[gi];
                if (d.kind == Engine::GateDesc::IDENTITY) continue;
                lgpu_fused_gate_t g{};
                g.ntgt = int32_t(d.tgts.size());
                for (size_t k = 0; k < d.tgts.size(); k++) g.tgt[k] = d.tgts[k];
                g.nctrl = int32_t(d.ctrls.size());
                for (size_t k = 0; k < d.ctrls.size(); k++) {
                    g.ctrl[k] = d.ctrls[k];
                    g.ctrl_val[k] = d.cvals.empty() ? 1 : d.cvals[k];
                }
                for (size_t e = 0; e < d.matrix.size(); e++) {
                    g.m[2 * e] = d.matrix[e].real();
                    g.m[2 * e + 1] = d.matrix[e].imag();
                }
                fg.push_back(g);
            }
            std::vector<int32_t> tb(blk.tile_bits.begin(), blk.tile_bits.end());
            const bool next_fused = bi + 1 < plan.size() && !plan[bi + 1].tile_bits.empty();
            const uint32_t ff = ff_ok ? ((in_ff ? LGPU_FF_IN : 0u) | (next_fused ? LGPU_FF_OUT : 0u)) : 0u;
            PL_LGPU_IS_SUCCESS(lgpu_apply_fused_block_ff(BaseType::getData(), nq(), dt(), uint32_t(tb.size()),
                                                         tb.data(), uint32_t(fg.size()), fg.data(), ff,
                                                         BaseType::lstream()));
            in_ff = ff_ok && next_fused;
        }
    }

    // ---- misc -------------------------------------------------------------------
    void sync() const {
        PL_LGPU_IS_SUCCESS(lgpu_stream_sync(BaseType::lstream()));
        int code = 0;
        PL_LGPU_IS_SUCCESS(lgpu_stream_error(BaseType::lstream(), &code, 1));
        PL_ABORT_IF(code != 0, "A GPU kernel timed out waiting for a bulk copy; the state is invalid");
    }
    lgpu_context_t ctx() const { return ctx_->get(); }
    static constexpr lgpu_dtype_t dt() { return cuUtil::dtype_of<Precision>(); }
    uint32_t nq() const { return uint32_t(BaseType::getNumQubits()); }
    auto getHandle() const -> CUDA::SharedCusvHandle { return handle_; }

    struct SparseDev {
        std::unique_ptr<CUDA::DataBuffer<int64_t, int>> off, col;
        std::unique_ptr<CUDA::DataBuffer<CFP_t, int>> val;
    };
    template <class index_type>
    SparseDev uploadCSR(const index_type *off, size_t noff, const index_type *cols, const std::complex<Precision> *vals,
                        size_t nnz) const {
        const auto dev = BaseType::getDataBuffer().getDevTag().getDeviceID();
        const auto stream = BaseType::getDataBuffer().getDevTag().getStreamID();
        std::vector<int64_t> o(off, off + noff), c(cols, cols + nnz);
        PL_ABORT_IF(noff < 1 || o.back() != int64_t(nnz), "Invalid CSR offsets");
        for (size_t r = 0; r + 1 < noff; r++) PL_ABORT_IF(o[r] > o[r + 1], "CSR offsets must be non-decreasing");
        for (auto x : c) PL_ABORT_IF(x < 0 || size_t(x) >= BaseType::getLength(), "CSR column index out of range");
        SparseDev sp;
        sp.off = std::make_unique<CUDA::DataBuffer<int64_t, int>>(noff, dev, stream, true);
        sp.col = std::make_unique<CUDA::DataBuffer<int64_t, int>>(std::max<size_t>(nnz, 1), dev, stream, true);
        sp.val = std::make_unique<CUDA::DataBuffer<CFP_t, int>>(std::max<size_t>(nnz, 1), dev, stream, true);
        sp.off->CopyHostDataToGpu(o.data(), noff, false);
        if (nnz) {
            sp.col->CopyHostDataToGpu(c.data(), nnz, false);
            sp.val->CopyHostDataToGpu(reinterpret_cast<const CFP_t *>(vals), nnz, false);
        }
        return sp;
    }

  private:
    static std::string key(const std::string &name, const std::vector<double> &p) {
        return name + "#" + std::to_string(p.empty() ? 0.0 : p[0]);
    }
    static bool known_gate(const std::string &name) {
        static const char *names[] = {"Identity", "I", "PauliX", "PauliY", "PauliZ", "Hadamard", "S", "T", "CNOT",
                                      "CY", "CZ", "SWAP", "CSWAP", "Toffoli", "RX", "RY", "RZ", "CRX", "CRY", "CRZ",
                                      "Rot", "CRot", "PhaseShift", "ControlledPhaseShift", "MultiRZ", "IsingXX",
                                      "IsingYY", "IsingZZ", "SingleExcitation", "SingleExcitationMinus",
                                      "SingleExcitationPlus", "DoubleExcitation", "DoubleExcitationMinus",
                                      "DoubleExcitationPlus"};
        for (const char *s : names)
            if (name == s) return true;
        return false;
    }
    void ctrl_last(const char *name, const std::vector<size_t> &wires, bool adjoint) {
        PL_ABORT_IF(wires.empty(), "Gate needs at least one wire");
        std::vector<cd> m;
        Engine::constant_gate(name, m);
        if (adjoint) m = Engine::dagger(m);
        std::vector<int> c;
        for (size_t k = 0; k + 1 < wires.size(); k++) {
            PL_ABORT_IF(wires[k] >= nq(), "Wire index out of range");
            c.push_back(Engine::bit_of(nq(), wires[k]));
        }
        PL_ABORT_IF(wires.back() >= nq(), "Wire index out of range");
        applyMatrixBits(m, {Engine::bit_of(nq(), wires.back())}, c, {});
    }
    void rot_last(const char *name, const std::vector<size_t> &wires, bool adjoint, Precision param) {
        PL_ABORT_IF(wires.empty(), "Gate needs at least one wire");
        using C = cuDoubleComplex;
        const double th = adjoint ? -double(param) : double(param);
        std::vector<cd> m = name[1] == 'X' ? Engine::to_cd(CUDA::cuGates::getRX<C>(th))
                            : name[1] == 'Y' ? Engine::to_cd(CUDA::cuGates::getRY<C>(th))
                                             : Engine::to_cd(CUDA::cuGates::getRZ<C>(th));
        std::vector<int> c;
        for (size_t k = 0; k + 1 < wires.size(); k++) {
            PL_ABORT_IF(wires[k] >= nq(), "Wire index out of range");
            c.push_back(Engine::bit_of(nq(), wires[k]));
        }
        PL_ABORT_IF(wires.back() >= nq(), "Wire index out of range");
        applyMatrixBits(m, {Engine::bit_of(nq(), wires.back())}, c, {});
    }
    void gen(const char *name, const std::vector<size_t> &wires, bool adjoint) {
        std::vector<int> bits;
        for (size_t w : wires) {
            PL_ABORT_IF(w >= nq(), "Wire index out of range");
            bits.push_back(Engine::bit_of(nq(), w));
        }
        std::vector<cd> g;
        double s = 0;
        PL_ABORT_IF_NOT(Engine::generator_of(name, bits.size(), g, s), "No generator");
        if (adjoint) g = Engine::dagger(g);
        applyMatrixBits(g, bits, {}, {});
    }

    CUDA::SharedCusvHandle handle_;
    std::shared_ptr<CUDA::LgpuContext> ctx_;
    std::optional<uint64_t> seed_;
    std::map<std::string, std::vector<cd>> user_gate_cache_;
    bool fusion_ = true;
    int fusion_tile_bits_ = 0;
    int fusion_min_low_bits_ = 0;
};

} // namespace Pennylane
