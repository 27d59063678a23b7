// fpa_devctx.h -- per-device library state, created on first use with that device current.
//
// The library's context (SM count for grid sizing, the device word the kernels report
// correction-loop errors into) belongs to one GPU.  A caller that switches devices with
// cudaSetDevice gets the state of the device current at the call; each device's entry is
// made once, by the first call that finds that device current.  Host-only code: the
// device query and the initialiser are passed in, so the keying is testable without a GPU.
#pragma once
#include <mutex>

template <class T, int MaxDevices = 64>
class PerDevice {
 public:
  // `query(int &dev)` returns false when no device can be named; `init(dev, T &)` fills a
  // new entry and returns false on failure (the entry then stays unset and is retried).
  template <class Query, class Init>
  bool get(Query query, Init init, T &out) {
    int dev = -1;
    if (!query(dev) || dev < 0 || dev >= MaxDevices) return false;
    std::lock_guard<std::mutex> lk(mu_);
    if (!ready_[dev]) {
      if (!init(dev, vals_[dev])) return false;
      ready_[dev] = true;
    }
    out = vals_[dev];
    return true;
  }
  // the entry of `dev` if it was made (no initialisation)
  bool peek(int dev, T &out) {
    if (dev < 0 || dev >= MaxDevices) return false;
    std::lock_guard<std::mutex> lk(mu_);
    if (!ready_[dev]) return false;
    out = vals_[dev];
    return true;
  }

 private:
  std::mutex mu_;
  bool ready_[MaxDevices] = {};
  T vals_[MaxDevices] = {};
};
