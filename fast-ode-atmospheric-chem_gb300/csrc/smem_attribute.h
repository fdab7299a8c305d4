// Per-device dynamic shared-memory limits of the library's kernels.
#pragma once

#include <cuda_runtime.h>

#include <mutex>

namespace fo {

// The dynamic shared-memory limit above 48 KB is an attribute of a kernel on
// one device: it is set once per (kernel, device) for the largest size asked
// so far, under a lock, so a process that drives several devices, or several
// host threads, never launches on a device where it was not set.
class SmemAttribute {
 public:
  explicit SmemAttribute(const void* kernel) : kernel_(kernel) {}
  cudaError_t ensure(size_t smem) {
    if (smem <= 48 * 1024) return cudaSuccess;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(mutex_);
    if ((int)smem <= configured_[dev]) return cudaSuccess;
    e = cudaFuncSetAttribute(kernel_, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess) configured_[dev] = (int)smem;
    return e;
  }

 private:
  static constexpr int kMaxDevices = 64;
  const void* kernel_;
  std::mutex mutex_;
  int configured_[kMaxDevices] = {};
};

}  // namespace fo
