// Per-device record of the dynamic shared memory each kernel has been allowed.
//
// cudaFuncSetAttribute(..., cudaFuncAttributeMaxDynamicSharedMemorySize, n) acts on
// the current device only, so a process that drives several GPUs (one engine per
// device, e.g. site shards) must raise it once on every device it launches on.  The
// allowance is only ever raised, never lowered: handles of different sizes share one
// kernel.  A mutex guards the record, so engines on different host threads may
// launch at the same time.  Raised by the layout's occupancy query and by the first,
// eager evaluation of a layout, never inside a stream capture.
#pragma once

#include <cuda_runtime.h>

#include <mutex>

namespace mcphy {

constexpr int kMaxDevices = 64;

class SmemAllowance {
  public:
    // Makes sure the kernel may use `bytes` of dynamic shared memory on `device`,
    // calling set(bytes) (which must act on that device) when the allowance
    // recorded for it is smaller.  A failed set leaves the record unchanged.
    template <typename Set>
    cudaError_t raise(int device, int bytes, Set set) {
        if (device < 0 || device >= kMaxDevices) return cudaErrorInvalidDevice;
        std::lock_guard<std::mutex> lock(mu_);
        if (bytes <= allowed_[device]) return cudaSuccess;
        const cudaError_t e = set(bytes);
        if (e == cudaSuccess) allowed_[device] = bytes;
        return e;
    }
    int allowed(int device) {
        if (device < 0 || device >= kMaxDevices) return 0;
        std::lock_guard<std::mutex> lock(mu_);
        return allowed_[device];
    }

  private:
    std::mutex mu_;
    int allowed_[kMaxDevices] = {};
};

// The same for the current device.
template <typename Set>
cudaError_t raise_smem(SmemAllowance& a, int bytes, Set set) {
    int dev = 0;
    const cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    return a.raise(dev, bytes, set);
}

}  // namespace mcphy
