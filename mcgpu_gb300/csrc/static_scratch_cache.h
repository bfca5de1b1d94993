// static_scratch_cache.h -- per-device cache of a __device__ array's address
// for mcgpu_system_energy_static, keyed on the identity of the CUDA context
// current when it was looked up.
//
// The address of a file-scope __device__ array is that of the module loaded
// into one context.  If the host application resets the device
// (cudaDeviceReset) or releases and re-creates its primary context, the
// module is loaded again, possibly at another address, and an address cached
// from the old context would send the next launch into memory that is no
// longer ours.  So each entry remembers the id of the context it was looked
// up in (cuCtxGetId: unique for the life of the process, even where a
// context handle is reused), and a call whose current context has another id
// looks the address up again.  Pure host code with the lookups passed in, so
// the refresh rule is unit-tested without a GPU.
#pragma once

#include <mutex>

namespace mcgpu {

template <int kMaxDevices>
class ScratchAddressCache {
 public:
  // Address of the scratch for `device` in the context whose id is
  // `ctx_id` (0: unknown, never matches a cached entry).  `lookup(void**)`
  // returns true and sets the address on success; `current_id()` gives the
  // context id after a lookup (the lookup may have created the context).
  // Returns nullptr if the lookup fails or the device index is out of range.
  template <class Lookup, class CurrentId>
  void* get(int device, unsigned long long ctx_id, Lookup lookup, CurrentId current_id) {
    if (device < 0 || device >= kMaxDevices) return nullptr;
    std::lock_guard<std::mutex> lock(mu_);
    Entry& e = entry_[device];
    if (e.addr && ctx_id != 0 && e.ctx_id == ctx_id) return e.addr;
    void* p = nullptr;
    if (!lookup(&p) || !p) {
      e = Entry();
      return nullptr;
    }
    e.addr = p;
    e.ctx_id = current_id();
    lookups_++;
    return p;
  }
  // Number of address lookups made so far (for tests).
  long long lookups() const { return lookups_; }

 private:
  struct Entry {
    void* addr = nullptr;
    unsigned long long ctx_id = 0;
  };
  std::mutex mu_;
  Entry entry_[kMaxDevices];
  long long lookups_ = 0;
};

}  // namespace mcgpu
