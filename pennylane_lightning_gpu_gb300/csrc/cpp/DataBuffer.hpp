// DataBuffer: RAII device allocation with host/device copies
// (reference src/util/DataBuffer.hpp:16-224).  All CUDA runtime work goes
// through the lgpu C ABI.
#pragma once

#include <cstddef>
#include <vector>

#include "DevTag.hpp"
#include "Error.hpp"

namespace Pennylane::CUDA {

template <class GPUDataT, class DevTagT = int> class DataBuffer {
  public:
    using type = GPUDataT;

    DataBuffer(std::size_t length, int device_id = 0, cudaStream_t stream_id = 0, bool alloc_memory = true)
        : length_{length}, dev_tag_{device_id, stream_id}, gpu_buffer_{nullptr} {
        if (alloc_memory && (length > 0)) {
            dev_tag_.refresh();
            PL_LGPU_IS_SUCCESS(lgpu_malloc_async(reinterpret_cast<void **>(&gpu_buffer_), sizeof(GPUDataT) * length,
                                                 lstream()));
        }
    }

    DataBuffer(std::size_t length, const DevTag<DevTagT> &dev, bool alloc_memory = true)
        : length_{length}, dev_tag_{dev}, gpu_buffer_{nullptr} {
        if (alloc_memory && (length > 0)) {
            dev_tag_.refresh();
            PL_LGPU_IS_SUCCESS(lgpu_malloc_async(reinterpret_cast<void **>(&gpu_buffer_), sizeof(GPUDataT) * length,
                                                 lstream()));
        }
    }

    DataBuffer(std::size_t length, DevTag<DevTagT> &&dev, bool alloc_memory = true)
        : length_{length}, dev_tag_{std::move(dev)}, gpu_buffer_{nullptr} {
        if (alloc_memory && (length > 0)) {
            dev_tag_.refresh();
            PL_LGPU_IS_SUCCESS(lgpu_malloc_async(reinterpret_cast<void **>(&gpu_buffer_), sizeof(GPUDataT) * length,
                                                 lstream()));
        }
    }

    DataBuffer() = delete;
    DataBuffer(const DataBuffer &) = delete;
    DataBuffer &operator=(const DataBuffer &) = delete;

    DataBuffer(DataBuffer &&other) noexcept
        : length_{other.length_}, dev_tag_{std::move(other.dev_tag_)}, gpu_buffer_{other.gpu_buffer_} {
        other.length_ = 0;
        other.gpu_buffer_ = nullptr;
    }
    DataBuffer &operator=(DataBuffer &&other) noexcept {
        if (this != &other) {
            if (gpu_buffer_) lgpu_free_async(gpu_buffer_, lstream());
            length_ = other.length_;
            dev_tag_ = std::move(other.dev_tag_);
            gpu_buffer_ = other.gpu_buffer_;
            other.length_ = 0;
            other.gpu_buffer_ = nullptr;
        }
        return *this;
    }

    virtual ~DataBuffer() {
        if (gpu_buffer_ != nullptr) lgpu_free_async(gpu_buffer_, lstream());
    }

    auto zeroInit() {
        PL_LGPU_IS_SUCCESS(lgpu_memset(gpu_buffer_, 0, length_ * sizeof(GPUDataT),
                                       reinterpret_cast<lgpu_stream_t>(dev_tag_.getStreamID())));
    }

    // stream-ordered allocation on this buffer's stream: no device-wide
    // synchronisation when states come and go (cudaFree would synchronise)
    lgpu_stream_t lstream() const { return reinterpret_cast<lgpu_stream_t>(dev_tag_.getStreamID()); }

    auto getData() -> GPUDataT * { return gpu_buffer_; }
    auto getData() const -> const GPUDataT * { return gpu_buffer_; }
    auto getLength() const { return length_; }
    auto getStream() const -> cudaStream_t { return dev_tag_.getStreamID(); }
    [[nodiscard]] inline auto getDevice() const -> int { return dev_tag_.getDeviceID(); }
    [[nodiscard]] inline auto getDevTag() const -> const DevTag<DevTagT> & { return dev_tag_; }

    template <class DataBufferT>
    void CopyGpuDataToGpu(const DataBufferT &buffer, bool async = false) {
        PL_ABORT_IF_NOT(buffer.getLength() == length_, "Sizes do not match for GPU data. Please ensure the "
                                                       "source buffer is not larger than the destination buffer");
        PL_LGPU_IS_SUCCESS(lgpu_memcpy(gpu_buffer_, buffer.getData(), sizeof(GPUDataT) * length_, LGPU_D2D,
                                       async ? 1 : 0, stream()));
    }

    void CopyGpuDataToGpu(const GPUDataT *gpu_in, std::size_t length, bool async = false) {
        PL_ABORT_IF_NOT(length == length_, "Sizes do not match for GPU data. Please ensure the source "
                                           "buffer is not larger than the destination buffer");
        PL_LGPU_IS_SUCCESS(lgpu_memcpy(gpu_buffer_, gpu_in, sizeof(GPUDataT) * length_, LGPU_D2D, async ? 1 : 0,
                                       stream()));
    }

    template <class HostDataT = GPUDataT>
    void CopyHostDataToGpu(const HostDataT *host_in, std::size_t length, bool async = false) {
        PL_ABORT_IF_NOT((sizeof(HostDataT) * length) <= (sizeof(GPUDataT) * length_),
                        "Sizes do not match for host & GPU data. Please ensure the source buffer is not larger "
                        "than the destination buffer");
        PL_LGPU_IS_SUCCESS(
            lgpu_memcpy(gpu_buffer_, host_in, sizeof(HostDataT) * length, LGPU_H2D, async ? 1 : 0, stream()));
    }

    template <class HostDataT = GPUDataT>
    void CopyGpuDataToHost(HostDataT *host_out, std::size_t length, bool async = false) const {
        PL_ABORT_IF_NOT((sizeof(HostDataT) * length) <= (sizeof(GPUDataT) * length_),
                        "Sizes do not match for host & GPU data. Please ensure the source buffer is not larger "
                        "than the destination buffer");
        PL_LGPU_IS_SUCCESS(
            lgpu_memcpy(host_out, gpu_buffer_, sizeof(HostDataT) * length, LGPU_D2H, async ? 1 : 0, stream()));
    }

  private:
    lgpu_stream_t stream() const { return reinterpret_cast<lgpu_stream_t>(dev_tag_.getStreamID()); }
    std::size_t length_;
    DevTag<DevTagT> dev_tag_;
    GPUDataT *gpu_buffer_;
};

} // namespace Pennylane::CUDA
