// Per-device one-time setup.  Settings such as cudaFuncSetAttribute belong to the
// context of the device that is current when they are made, so a process that launches
// on several devices must make them once on each.
#pragma once
#include <cuda_runtime.h>

#include <mutex>
#include <utility>

namespace rc {

constexpr int kOnceDevices = 64;

// Runs f once for the current device (every time if the device cannot be identified).
template <class F>
void once_per_device(std::once_flag (&flags)[kOnceDevices], F&& f) {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kOnceDevices) {
        f();
        return;
    }
    std::call_once(flags[dev], std::forward<F>(f));
}

}  // namespace rc
