// Once-per-device initialisation (function attributes, symbol addresses):
// CUDA keeps such settings per device, so a process that uses several GPUs
// must repeat them on each.  Thread-safe; a failed initialisation is retried
// on the next call.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <mutex>
#include <stdint.h>

namespace fgb {

struct PerDeviceOnce {
  std::atomic<uint64_t> done{0};  // bit d: device d initialised
  std::mutex mu;

  // Runs init() with the current device current, unless it already succeeded
  // on that device.  Devices beyond 63 run init() on every call.
  template <class F>
  cudaError_t run(F&& init) {
    int dev = 0;
    const cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 64) return init();
    const uint64_t bit = uint64_t(1) << dev;
    if (done.load(std::memory_order_acquire) & bit) return cudaSuccess;
    std::lock_guard<std::mutex> lock(mu);
    if (done.load(std::memory_order_relaxed) & bit) return cudaSuccess;
    const cudaError_t r = init();
    if (r == cudaSuccess) done.fetch_or(bit, std::memory_order_release);
    return r;
  }
};

// Restores the calling thread's current device when it goes out of scope.
class DeviceGuard {
 public:
  DeviceGuard() { ok_ = cudaGetDevice(&dev_) == cudaSuccess; }
  ~DeviceGuard() {
    if (ok_) cudaSetDevice(dev_);
  }
  DeviceGuard(const DeviceGuard&) = delete;
  DeviceGuard& operator=(const DeviceGuard&) = delete;

 private:
  int dev_ = 0;
  bool ok_ = false;
};

}  // namespace fgb
