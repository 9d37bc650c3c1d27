// per_device.h -- one-time launch set-up kept per device ordinal.
//
// A kernel's MaxDynamicSharedMemorySize attribute applies to the device that
// was current when it was set, and a persistent grid is sized from that
// device's SM count and occupancy.  Neither may be cached once per process:
// a process that drives tiles on two GPUs would launch on the second one
// without the attribute (a launch failure for > 48 KB of dynamic shared
// memory) or with the first one's grid.  PerDevice keeps one value per
// device ordinal instead.
//
// Plain C++ (no CUDA types), so that the lookup is testable on a host
// without a GPU through a fake device ordinal and a fake set-up function.
#pragma once
#include <atomic>

namespace ocean {

constexpr int kMaxDevices = 64;   // device ordinals the caches hold

// One int per device ordinal; 0 means "not set up yet", so a set-up must
// produce a non-zero value (a grid size, or 1 for "attribute set").
class PerDevice {
public:
    // The value of device `dev`, running `init(&value)` on the first request
    // for that device.  init returns 0 on success or an error code, which is
    // returned unchanged (nothing is cached then, so a later call retries).
    // Threads racing on the first request of one device all run init; each
    // applies the same device setting and stores the same value.
    // Returns `bad_device` for ordinals outside [0, kMaxDevices).
    template <class Init>
    int get(int dev, int* value, int bad_device, Init&& init)
    {
        if (dev < 0 || dev >= kMaxDevices) return bad_device;
        int v = slot_[dev].load(std::memory_order_acquire);
        if (v == 0) {
            const int rc = init(&v);
            if (rc != 0) return rc;
            if (v == 0) return bad_device;
            slot_[dev].store(v, std::memory_order_release);
        }
        *value = v;
        return 0;
    }

private:
    std::atomic<int> slot_[kMaxDevices] = {};
};

}  // namespace ocean
