// CPU test of the C ABI's current-device guard (simit_gb300/csrc/
// sg_device_guard.h) with a fake device API: the context's device is made
// current for the call and the caller's device comes back afterwards,
// including on an early return; nothing changes when they already agree or
// when the device cannot be queried.
#include <cstdio>
#include <cstdlib>

#include "../../simit_gb300/csrc/sg_device_guard.h"

namespace {
int g_cur = 0, g_sets = 0;
bool g_get_ok = true;
struct FakeApi {
  static bool get(int *d) {
    if (!g_get_ok) return false;
    *d = g_cur;
    return true;
  }
  static bool set(int d) {
    g_cur = d;
    ++g_sets;
    return true;
  }
};
using Guard = sg::DeviceGuardT<FakeApi>;

#define CHECK(c)                                              \
  do {                                                        \
    if (!(c)) {                                               \
      std::fprintf(stderr, "%s:%d: %s\n", __FILE__, __LINE__, #c); \
      std::exit(1);                                           \
    }                                                         \
  } while (0)

int entry_point(int ctx_device, bool early, int *seen) {
  Guard g(ctx_device);
  *seen = g_cur;
  if (early) return -1;
  return 0;
}
}  // namespace

int main() {
  int seen = -1;
  g_cur = 0;
  entry_point(1, false, &seen);
  CHECK(seen == 1 && g_cur == 0 && g_sets == 2);
  entry_point(3, true, &seen);  // early return still restores
  CHECK(seen == 3 && g_cur == 0 && g_sets == 4);
  g_cur = 2;
  entry_point(2, false, &seen);  // same device: no switch
  CHECK(seen == 2 && g_cur == 2 && g_sets == 4);
  entry_point(-1, false, &seen);  // no context: no switch
  CHECK(g_cur == 2 && g_sets == 4);
  g_get_ok = false;
  entry_point(0, false, &seen);  // device unknown: left alone
  CHECK(g_cur == 2 && g_sets == 4);
  {
    g_get_ok = true;
    Guard outer(5);
    CHECK(g_cur == 5);
    {
      Guard inner(6);
      CHECK(g_cur == 6);
    }
    CHECK(g_cur == 5);
  }
  CHECK(g_cur == 2);
  std::printf("device guard ok\n");
  return 0;
}
