// Complex-number helpers, device queries and engine handles
// (reference src/util/cuda_helpers.hpp).  The reference's cuBLAS / cuSPARSE /
// cuStateVec handles become one opaque engine handle type; the constructor
// arguments that took them keep their positions and defaults.
#pragma once

#include <cuComplex.h>
#include <cuda_runtime_api.h>

#include <complex>
#include <memory>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include "Error.hpp"

namespace Pennylane::CUDA::Util {

template <class T> inline static constexpr auto ConstMult(T a, T b) -> T {
    return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x};
}
template <class T> inline static constexpr auto ConstSum(T a, T b) -> T { return {a.x + b.x, a.y + b.y}; }
template <class T, class U> inline static constexpr auto ConstMultSC(U a, T b) -> T { return {a * b.x, a * b.y}; }
template <class T> inline static constexpr auto ONE() -> T { return {1, 0}; }
template <class T> inline static constexpr auto ZERO() -> T { return {0, 0}; }
template <class T> inline static constexpr auto IMAG() -> T { return {0, 1}; }
template <class T> inline static constexpr auto SQRT2() {
    if constexpr (std::is_same_v<T, float2> || std::is_same_v<T, cuFloatComplex>) {
        return T{0x1.6a09e6p+0F, 0};
    } else if constexpr (std::is_same_v<T, double2> || std::is_same_v<T, cuDoubleComplex>) {
        return T{0x1.6a09e667f3bcdp+0, 0};
    } else if constexpr (std::is_same_v<T, double>) {
        return 0x1.6a09e667f3bcdp+0;
    } else {
        return 0x1.6a09e6p+0F;
    }
}
template <class T> inline static constexpr auto INVSQRT2() -> T {
    if constexpr (std::is_same_v<T, std::complex<float>> || std::is_same_v<T, std::complex<double>>) {
        return T(1 / M_SQRT2);
    } else {
        return {static_cast<decltype(T{}.x)>(1 / M_SQRT2), 0};
    }
}

template <class T> inline auto complexToCu(T a) {
    if constexpr (std::is_same_v<T, std::complex<double>>) {
        return make_cuDoubleComplex(a.real(), a.imag());
    } else {
        return make_cuFloatComplex(a.real(), a.imag());
    }
}
template <class T, class U = double> inline auto cuToComplex(T a) -> std::complex<U> {
    return std::complex<U>{a.x, a.y};
}

inline cuDoubleComplex getCudaType(const double &t) {
    static_cast<void>(t);
    return {};
}
inline cuFloatComplex getCudaType(const float &t) {
    static_cast<void>(t);
    return {};
}

// lgpu dtype of a precision
template <class P> constexpr lgpu_dtype_t dtype_of() {
    return std::is_same_v<P, double> ? LGPU_C128 : LGPU_C64;
}

inline int getGPUCount() {
    int result = 0;
    if (lgpu_device_count(&result) != LGPU_OK) return 0;
    return result;
}
inline int getGPUIdx() {
    int result = 0;
    PL_LGPU_IS_SUCCESS(lgpu_get_device(&result));
    return result;
}
inline void deviceReset() { PL_LGPU_IS_SUCCESS(lgpu_device_reset()); }

// The engine is written for sm_103a; any device of compute capability >= 10
// loads its cubins only when it is exactly that architecture.
inline std::pair<int, int> getGPUArch(int device_number = 0) {
    int major = 0, minor = 0;
    PL_LGPU_IS_SUCCESS(lgpu_device_arch(device_number, &major, &minor));
    return {major, minor};
}
inline bool isCuQuantumSupported(int device_number = 0) {
    int count = getGPUCount();
    if (device_number >= count) return false;
    auto [major, minor] = getGPUArch(device_number);
    return major == 10 && minor == 3;
}

// Pauli letter -> integer (reference cuda_helpers.hpp:680-703 maps to
// custatevecPauli_t; here the engine takes bit masks).
inline std::vector<int> pauliStringToEnum(const std::string &pauli_word) {
    std::vector<int> out;
    for (char c : pauli_word) {
        switch (c) {
        case 'I': out.push_back(0); break;
        case 'X': out.push_back(1); break;
        case 'Y': out.push_back(2); break;
        case 'Z': out.push_back(3); break;
        default: PL_ABORT("Invalid character in Pauli word");
        }
    }
    return out;
}

} // namespace Pennylane::CUDA::Util

namespace Pennylane::CUDA {

// Opaque engine handle (stands in for custatevecHandle_t / cublasHandle_t /
// cusparseHandle_t in the reference's constructor signatures).  Each state
// vector keeps its own scratch context, so handles only carry the device.
struct EngineHandle {
    int device = 0;
};
using SharedCusvHandle = std::shared_ptr<EngineHandle>;
using SharedCublasCaller = std::shared_ptr<EngineHandle>;
using SharedCusparseHandle = std::shared_ptr<EngineHandle>;
inline SharedCusvHandle make_shared_cusv_handle() { return std::make_shared<EngineHandle>(); }
inline SharedCublasCaller make_shared_cublas_caller() { return std::make_shared<EngineHandle>(); }
inline SharedCusparseHandle make_shared_cusparse_handle() { return std::make_shared<EngineHandle>(); }

// RAII lgpu scratch context (one per state vector / algorithm instance).
class LgpuContext {
  public:
    // contexts come from (and return to) the library's per-device free list;
    // the owner finishes the work that uses the context before it is released
    explicit LgpuContext(int device = 0) { PL_LGPU_IS_SUCCESS(lgpu_context_acquire(device, &ctx_)); }
    ~LgpuContext() { lgpu_context_release(ctx_); }
    LgpuContext(const LgpuContext &) = delete;
    LgpuContext &operator=(const LgpuContext &) = delete;
    lgpu_context_t get() const { return ctx_; }

  private:
    lgpu_context_t ctx_ = nullptr;
};

} // namespace Pennylane::CUDA

namespace cuUtil = Pennylane::CUDA::Util;
