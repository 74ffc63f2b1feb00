// device_buffers.h -- one owner for a set of device allocations: freed together when the
// owner goes away, released one by one when replaced, their bytes counted.
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <vector>

namespace fe {

class DeviceBuffers {
public:
    DeviceBuffers() = default;
    DeviceBuffers(const DeviceBuffers&) = delete;
    DeviceBuffers& operator=(const DeviceBuffers&) = delete;
    ~DeviceBuffers() {
        for (const Buf& b : bufs_) cudaFree(b.p);
    }

    // count elements of T (at least one, so every buffer has an address)
    template <typename T>
    cudaError_t alloc(T** p, size_t count) {
        if (count == 0) count = 1;
        const cudaError_t e = cudaMalloc((void**)p, count * sizeof(T));
        if (e == cudaSuccess) {
            bufs_.push_back({(void*)*p, (int64_t)(count * sizeof(T))});
            bytes_ += (int64_t)(count * sizeof(T));
        }
        return e;
    }

    // alloc, then copy count elements from host memory (src may be null: no copy)
    template <typename T>
    cudaError_t upload(T** p, const T* src, size_t count) {
        cudaError_t e = alloc(p, count);
        if (e == cudaSuccess && src && count) e = cudaMemcpy(*p, src, count * sizeof(T), cudaMemcpyHostToDevice);
        return e;
    }

    // free one buffer made by alloc / upload
    void release(void* p) {
        for (size_t k = 0; k < bufs_.size(); ++k)
            if (bufs_[k].p == p) {
                cudaFree(p);
                bytes_ -= bufs_[k].bytes;
                bufs_.erase(bufs_.begin() + (long)k);
                return;
            }
    }

    int64_t bytes() const { return bytes_; }

private:
    struct Buf {
        void* p;
        int64_t bytes;
    };
    std::vector<Buf> bufs_;
    int64_t bytes_ = 0;
};

}  // namespace fe
