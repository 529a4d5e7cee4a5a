// Scoped current-device switch for the C ABI's entry points.
//
// A context belongs to one device; its stream, its per-device one-time set-up
// (function attributes, occupancy) and its allocations are only valid with
// that device current.  The runtime's current device is per host thread, so
// an entry point called from a thread whose current device differs (a
// context created on device 1, used from a thread that last used device 0)
// makes the context's device current for the duration of the call and
// restores the caller's device on return.  The device calls come from a
// policy (Api) so the logic can be tested without a GPU.
#pragma once

namespace sg {

template <class Api> class DeviceGuardT {
 public:
  explicit DeviceGuardT(int device) {
    if (device < 0) return;
    int cur = -1;
    if (!Api::get(&cur)) return;
    if (cur == device) return;
    if (Api::set(device)) {
      prev_ = cur;
      changed_ = true;
    }
  }
  ~DeviceGuardT() {
    if (changed_) Api::set(prev_);
  }
  DeviceGuardT(const DeviceGuardT &) = delete;
  DeviceGuardT &operator=(const DeviceGuardT &) = delete;
  bool changed() const { return changed_; }

 private:
  int prev_ = -1;
  bool changed_ = false;
};

}  // namespace sg
