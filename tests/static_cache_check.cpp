// Unit check of the scratch-address cache of mcgpu_system_energy_static
// (mcgpu_gb300/csrc/static_scratch_cache.h) with fake lookups: no GPU.
#include <cstdio>

#include "static_scratch_cache.h"

#define EXPECT(c)                                              \
  do {                                                         \
    if (!(c)) {                                                \
      std::printf("FAILED line %d: %s\n", __LINE__, #c);       \
      return 1;                                                \
    }                                                          \
  } while (0)

int main() {
  mcgpu::ScratchAddressCache<4> cache;
  static char mem_a[16], mem_b[16];
  void* where = mem_a;         // the module's current load address
  unsigned long long ctx = 7;  // the current context's id
  int calls = 0;
  auto lookup = [&](void** p) { calls++; *p = where; return true; };
  auto cur = [&]() { return ctx; };
  // first call looks up, the next ones in the same context do not
  EXPECT(cache.get(0, ctx, lookup, cur) == mem_a);
  EXPECT(cache.get(0, ctx, lookup, cur) == mem_a);
  EXPECT(calls == 1);
  // a device reset: new context id, module reloaded elsewhere
  ctx = 8;
  where = mem_b;
  EXPECT(cache.get(0, ctx, lookup, cur) == mem_b);
  EXPECT(calls == 2);
  EXPECT(cache.get(0, ctx, lookup, cur) == mem_b);
  EXPECT(calls == 2);
  // devices are cached separately
  EXPECT(cache.get(1, ctx, lookup, cur) == mem_b);
  EXPECT(calls == 3);
  // an unknown context id (0) never trusts the cache
  EXPECT(cache.get(0, 0, lookup, cur) == mem_b);
  EXPECT(calls == 4);
  // no context before the lookup: the id after it is cached
  mcgpu::ScratchAddressCache<4> c2;
  ctx = 11;
  EXPECT(c2.get(2, 0, lookup, cur) == mem_b);
  EXPECT(c2.get(2, 11, lookup, cur) == mem_b);
  EXPECT(calls == 5);
  // a failed lookup returns null and clears the entry
  auto bad = [&](void** p) { calls++; *p = nullptr; return false; };
  ctx = 12;
  EXPECT(cache.get(0, ctx, bad, cur) == nullptr);
  EXPECT(cache.get(0, ctx, lookup, cur) == mem_b);
  // out-of-range device index
  EXPECT(cache.get(4, ctx, lookup, cur) == nullptr);
  EXPECT(cache.get(-1, ctx, lookup, cur) == nullptr);
  std::printf("ok\n");
  return 0;
}
