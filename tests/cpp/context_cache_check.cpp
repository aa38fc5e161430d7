// Checks the per-device, per-context cache that holds the device address of
// the library's static scratch array (csrc/context_cache.h): a value is
// looked up once per device and context, looked up again when the device's
// context changes (as after cudaDeviceReset), kept per device, and not
// cached when the lookup fails. Exit status 0 = all checks passed.
#include "../../lippmann_schwinger_solver_gb300/csrc/context_cache.h"

#include <cstdio>

int main() {
  lsg::ContextCache<long> cache;
  int fails = 0;
  long next = 100;
  auto fetch = [&next](long* v) { *v = next++; return 0; };
  auto check = [&fails](bool ok, const char* what) {
    if (!ok) {
      std::printf("FAIL: %s\n", what);
      ++fails;
    }
  };
  long v = 0;
  check(cache.get(0, 7, fetch, &v) == 0 && v == 100, "first lookup on device 0");
  check(cache.get(0, 7, fetch, &v) == 0 && v == 100 && cache.fetches() == 1, "same context reuses the value");
  check(cache.get(0, 8, fetch, &v) == 0 && v == 101 && cache.fetches() == 2, "new context looks it up again");
  check(cache.get(0, 8, fetch, &v) == 0 && v == 101, "then keeps the new value");
  check(cache.get(1, 8, fetch, &v) == 0 && v == 102, "devices have their own slots");
  check(cache.get(0, 8, fetch, &v) == 0 && v == 101, "device 0 unchanged by device 1");
  check(cache.get(0, 7, fetch, &v) == 0 && v == 103, "returning to an old context ID looks it up again");
  auto failing = [](long* out) { *out = -5; return 17; };
  check(cache.get(2, 1, failing, &v) == 17, "a failed lookup passes its code back");
  check(cache.get(2, 1, fetch, &v) == 0 && v == 104, "and caches nothing");
  check(cache.get(-1, 1, fetch, &v) == -1 && cache.get(64, 1, fetch, &v) == -1, "device index out of range");
  std::printf("context cache checks: %d failed\n", fails);
  return fails ? 1 : 0;
}
