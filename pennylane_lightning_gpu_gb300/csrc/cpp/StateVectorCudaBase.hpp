// Base class of the device state vector: owns the 2^n amplitude buffer and
// provides host/device copies and |0...0> initialisation (reference
// src/simulator/StateVectorCudaBase.hpp:54-313, CRTP over the derived class).
#pragma once

#include <complex>
#include <memory>
#include <string>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include "DataBuffer.hpp"
#include "cuda_helpers.hpp"

namespace Pennylane {

namespace Util {
inline constexpr size_t exp2(size_t n) { return size_t(1) << n; }
inline size_t log2(size_t value) {
    size_t r = 0;
    while ((size_t(1) << r) < value) r++;
    return r;
}
} // namespace Util

template <class PrecisionT, class Derived> class StateVectorCudaBase {
  public:
    using scalar_type_t = PrecisionT;
    using CFP_t = decltype(cuUtil::getCudaType(PrecisionT{}));

    StateVectorCudaBase() = delete;
    StateVectorCudaBase(size_t num_qubits, int device_id = 0, cudaStream_t stream_id = 0, bool device_alloc = true)
        : num_qubits_{num_qubits},
          data_buffer_{std::make_unique<CUDA::DataBuffer<CFP_t>>(Util::exp2(num_qubits), device_id, stream_id,
                                                                 device_alloc)} {
        check_size(num_qubits);
    }
    StateVectorCudaBase(size_t num_qubits, CUDA::DevTag<int> dev_tag, bool device_alloc = true)
        : num_qubits_{num_qubits},
          data_buffer_{std::make_unique<CUDA::DataBuffer<CFP_t>>(Util::exp2(num_qubits), dev_tag, device_alloc)} {
        check_size(num_qubits);
    }
    virtual ~StateVectorCudaBase() = default;

    [[nodiscard]] auto getNumQubits() const -> size_t { return num_qubits_; }
    [[nodiscard]] auto getLength() const -> size_t { return Util::exp2(num_qubits_); }
    [[nodiscard]] auto getData() -> CFP_t * { return data_buffer_->getData(); }
    [[nodiscard]] auto getData() const -> const CFP_t * { return data_buffer_->getData(); }
    [[nodiscard]] auto getStream() const -> cudaStream_t { return data_buffer_->getStream(); }
    auto getDataBuffer() -> CUDA::DataBuffer<CFP_t> & { return *data_buffer_; }
    auto getDataBuffer() const -> const CUDA::DataBuffer<CFP_t> & { return *data_buffer_; }
    lgpu_stream_t lstream() const { return reinterpret_cast<lgpu_stream_t>(getStream()); }

    void CopyHostDataToGpu(const std::vector<std::complex<PrecisionT>> &sv, bool async = false) {
        PL_ABORT_IF_NOT(getLength() == sv.size(), "Sizes do not match for Host and GPU data");
        data_buffer_->CopyHostDataToGpu(sv.data(), sv.size(), async);
    }
    void CopyHostDataToGpu(const std::complex<PrecisionT> *host_sv, size_t length, bool async = false) {
        PL_ABORT_IF_NOT(getLength() == length, "Sizes do not match for Host and GPU data");
        data_buffer_->CopyHostDataToGpu(reinterpret_cast<const CFP_t *>(host_sv), length, async);
    }
    void CopyGpuDataToGpuIn(const CFP_t *gpu_sv, size_t length, bool async = false) {
        PL_ABORT_IF_NOT(getLength() == length, "Sizes do not match for Host and GPU data");
        data_buffer_->CopyGpuDataToGpu(gpu_sv, length, async);
    }
    void CopyGpuDataToGpuIn(const Derived &sv, bool async = false) {
        PL_ABORT_IF_NOT(getNumQubits() == sv.getNumQubits(), "Sizes do not match for Host and GPU data");
        data_buffer_->CopyGpuDataToGpu(sv.getData(), sv.getLength(), async);
    }
    void CopyGpuDataToHost(std::complex<PrecisionT> *host_sv, size_t length, bool async = false) const {
        PL_ABORT_IF_NOT(getLength() == length, "Sizes do not match for Host and GPU data");
        data_buffer_->CopyGpuDataToHost(reinterpret_cast<CFP_t *>(host_sv), length, async);
    }
    void CopyGpuDataToGpuOut(Derived &sv, bool async = false) {
        PL_ABORT_IF_NOT(getNumQubits() == sv.getNumQubits(), "Sizes do not match for Host and GPU data");
        sv.getDataBuffer().CopyGpuDataToGpu(getData(), getLength(), async);
    }

    void updateData(const Derived &other, bool async = false) { CopyGpuDataToGpuIn(other, async); }
    void updateData(std::unique_ptr<CUDA::DataBuffer<CFP_t>> &&other) { data_buffer_ = std::move(other); }

    // |0...0>  (initSV.cu / StateVectorCudaBase.hpp:234-240)
    void initSV(bool async = false) {
        PL_LGPU_IS_SUCCESS(lgpu_set_basis(getData(), uint32_t(num_qubits_), cuUtil::dtype_of<PrecisionT>(), 0, 1.0,
                                          0.0, lstream()));
        if (!async) PL_LGPU_IS_SUCCESS(lgpu_stream_sync(lstream()));
    }

    // Control-wire counts per gate name (StateVectorCudaBase.hpp:288-312).
    auto getCtrlMap() const -> const std::unordered_map<std::string, std::size_t> & { return ctrl_map_; }
    auto getConstGates() const -> const std::unordered_set<std::string> & { return const_gates_; }

  protected:
    static void check_size(size_t n) {
        PL_ABORT_IF(n < 1 || n > LGPU_MAX_QUBITS, "Number of qubits must be between 1 and 34");
    }

  private:
    size_t num_qubits_;
    std::unique_ptr<CUDA::DataBuffer<CFP_t>> data_buffer_;
    const std::unordered_set<std::string> const_gates_{"Identity", "PauliX", "PauliY", "PauliZ", "Hadamard",
                                                       "T",        "S",      "CNOT",   "SWAP",   "CY",
                                                       "CZ",       "CSWAP",  "Toffoli"};
    const std::unordered_map<std::string, std::size_t> ctrl_map_{
        {"Identity", 0}, {"PauliX", 0}, {"PauliY", 0}, {"PauliZ", 0}, {"Hadamard", 0}, {"T", 0},
        {"S", 0},        {"RX", 0},     {"RY", 0},     {"RZ", 0},     {"Rot", 0},      {"PhaseShift", 0},
        {"ControlledPhaseShift", 1},    {"CNOT", 1},   {"SWAP", 0},   {"CY", 1},       {"CZ", 1},
        {"CRX", 1},      {"CRY", 1},    {"CRZ", 1},    {"CRot", 1},   {"CSWAP", 1},    {"Toffoli", 2}};
};

} // namespace Pennylane
