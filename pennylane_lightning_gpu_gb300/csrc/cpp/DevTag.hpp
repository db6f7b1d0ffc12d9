// DevTag: (device id, stream) pair carried by every buffer and state vector
// (reference src/util/DevTag.hpp:17-56).
#pragma once

#include <cuda_runtime_api.h>

#include "Error.hpp"

namespace Pennylane::CUDA {

template <class IDType> class DevTag {
  public:
    DevTag() : device_id_{0}, stream_id_{0} {}
    DevTag(IDType device_id) : device_id_{device_id}, stream_id_{0} {}
    DevTag(IDType device_id, cudaStream_t stream_id) : device_id_{device_id}, stream_id_{stream_id} {}
    DevTag(const DevTag &other) = default;
    DevTag(DevTag &&other) noexcept = default;
    DevTag &operator=(const DevTag &) = default;
    DevTag &operator=(DevTag &&) noexcept = default;
    virtual ~DevTag() = default;

    [[nodiscard]] inline auto getDeviceID() const -> IDType { return device_id_; }
    [[nodiscard]] inline auto getStreamID() const -> cudaStream_t { return stream_id_; }
    inline void refresh() { PL_LGPU_IS_SUCCESS(lgpu_set_device(static_cast<int>(device_id_))); }

  private:
    IDType device_id_;
    cudaStream_t stream_id_;
};

} // namespace Pennylane::CUDA
