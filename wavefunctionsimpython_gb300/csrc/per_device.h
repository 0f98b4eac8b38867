// per_device.h — values kept once per CUDA device.
//
// Function attributes set with cudaFuncSetAttribute (maximum dynamic shared
// memory, non-portable cluster sizes, carveout) and the occupancy figures derived
// from them belong to the device a kernel is launched on. A process that drives
// several GPUs, or several engines on different devices, must set them on each
// device; a process-wide "done" flag would skip the setting on the second device
// and its launches would fail. PerDevice keeps one int per device ordinal: 0
// means "not yet set". Two threads that race on a device's first launch both set
// the same attributes and store the same value, which is harmless.
#pragma once

#include <cuda_runtime.h>

#include <atomic>

namespace wfs {

struct PerDevice {
    static constexpr int kMaxDevices = 64;
    std::atomic<int> v[kMaxDevices];
    int get(int dev) const { return (dev >= 0 && dev < kMaxDevices) ? v[dev].load(std::memory_order_acquire) : 0; }
    void put(int dev, int x) {
        if (dev >= 0 && dev < kMaxDevices) v[dev].store(x, std::memory_order_release);
    }
};

inline int current_device() {
    int d = -1;
    return cudaGetDevice(&d) == cudaSuccess ? d : -1;
}

}  // namespace wfs
