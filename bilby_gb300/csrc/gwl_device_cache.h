// A process-wide table of per-device objects keyed by (CUDA device, key).
//
// Device allocations belong to the device that was current when they were
// made; a table shared by every device of the process must therefore key on
// the device as well as on what the object describes (an FFT length), or a
// launch on one GPU would read another GPU's memory.  Entries are created
// once, under the lock, and never replaced or freed while the process runs,
// so a pointer handed out stays valid for kernels in flight on any thread.
// Plain C++ (no CUDA headers), so that the keying can be tested on a host.
#pragma once

#include <cstdint>
#include <map>
#include <mutex>
#include <utility>

namespace gwl {

template <class V>
class PerDeviceCache {
 public:
  // The entry of (device, key): found, or made by `make(V*)`, which returns
  // 0 on success (the entry is then kept) or an error code (nothing is kept).
  template <class Make>
  int get(int device, int64_t key, V* out, Make make) {
    std::lock_guard<std::mutex> g(mu_);
    auto it = map_.find(std::make_pair(device, key));
    if (it != map_.end()) {
      *out = it->second;
      return 0;
    }
    V v{};
    const int rc = make(&v);
    if (rc) return rc;
    map_.emplace(std::make_pair(device, key), v);
    *out = v;
    return 0;
  }

  size_t size() {
    std::lock_guard<std::mutex> g(mu_);
    return map_.size();
  }

 private:
  std::mutex mu_;
  std::map<std::pair<int, int64_t>, V> map_;
};

}  // namespace gwl
