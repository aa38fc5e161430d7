// Per-device cache of a value that belongs to a CUDA context, such as the
// device address of a file-scope __device__ array: that address is only
// valid in the context it was looked up in. A device's context can change
// under a long-lived library (cudaDeviceReset destroys the primary context,
// and the next runtime call on that device creates a new one), so each
// entry remembers the context's unique ID and is looked up again when the
// current context has another one.
//
// Host-only and free of CUDA headers, so that the cache logic can be tested
// without a GPU.
#pragma once

#include <mutex>

namespace lsg {

template <class V, int MaxDevices = 64>
class ContextCache {
 public:
  // The value for `device` in the context with ID ctx_id: the cached one
  // when it was looked up in that same context, otherwise fetch(&v), which
  // returns 0 on success (any other code is passed back and nothing is
  // cached). Thread-safe.
  template <class Fetch>
  int get(int device, unsigned long long ctx_id, Fetch fetch, V* out) {
    if (device < 0 || device >= MaxDevices) return -1;
    std::lock_guard<std::mutex> lock(mu_);
    Slot& s = slots_[device];
    if (!s.valid || s.ctx_id != ctx_id) {
      V v{};
      const int rc = fetch(&v);
      if (rc != 0) return rc;
      s.value = v;
      s.ctx_id = ctx_id;
      s.valid = true;
      ++fetches_;
    }
    *out = s.value;
    return 0;
  }
  long long fetches() const { return fetches_; }

 private:
  struct Slot {
    unsigned long long ctx_id = 0;
    V value{};
    bool valid = false;
  };
  std::mutex mu_;
  Slot slots_[MaxDevices];
  long long fetches_ = 0;
};

}  // namespace lsg
