// launch_attr.h -- kernel attributes that must be set once per device before
// a kernel's first launch there (function attributes belong to a device).
#pragma once
#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>

namespace poe {

// raise kernel's dynamic shared-memory limit to bytes on the current device,
// once per device; done is the caller's per-kernel mask of devices (64 at most)
template <typename Kernel>
inline void smem_attr_once(Kernel kernel, int bytes, std::atomic<uint64_t> &done)
{
    int dev = 0;
    cudaGetDevice(&dev);
    const uint64_t bit = 1ull << (dev & 63);
    if (done.load(std::memory_order_acquire) & bit) return;
    cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    done.fetch_or(bit, std::memory_order_acq_rel);
}

}  // namespace poe
