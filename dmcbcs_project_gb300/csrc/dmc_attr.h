// Per-device record of the kernel attributes the library has set.
//
// cudaFuncSetAttribute acts on the current device only.  A context records
// the device it was created on, and contexts on different devices may run
// on different host threads at the same time, so the record of which
// dynamic shared-memory size (and carveout) a kernel has been opted into is
// kept per device and guarded by a mutex.  Plain C++ (no CUDA), so the
// bookkeeping is testable on a machine without a GPU.
#pragma once

#include <mutex>

namespace dmc {

class AttrCache {
public:
    static constexpr int kMaxDevices = 64;
    static constexpr int kKinds = 8;

    // Make sure attribute `kind` of device `dev` holds at least `value`:
    // calls set(value) (0 = success) unless the device already has a value
    // >= `value` recorded; the value is recorded only when set succeeds.
    // Devices or kinds outside the table are never cached (set runs every
    // time).  Returns set's result, or 0 when nothing had to be set.
    template <class F>
    int ensure(int dev, int kind, int value, F&& set)
    {
        if (dev < 0 || dev >= kMaxDevices || kind < 0 || kind >= kKinds) return set(value);
        std::lock_guard<std::mutex> g(mu_);
        if (have_[dev][kind] >= value) return 0;
        const int e = set(value);
        if (e == 0) have_[dev][kind] = value;
        return e;
    }

    // recorded value (-1: never set) -- for tests
    int recorded(int dev, int kind)
    {
        if (dev < 0 || dev >= kMaxDevices || kind < 0 || kind >= kKinds) return -1;
        std::lock_guard<std::mutex> g(mu_);
        return have_[dev][kind];
    }

    AttrCache()
    {
        for (auto& d : have_)
            for (int& k : d) k = -1;
    }

private:
    std::mutex mu_;
    int have_[kMaxDevices][kKinds];
};

}  // namespace dmc
