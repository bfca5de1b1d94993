// initial_config.cpp -- host-side initial configuration: molecule centres by
// random sequential addition with a minimum separation.  The reference builds
// its initial boxes on the host too (an FCC lattice, FileUtilities.cpp:
// 550-642); this builder places centres uniformly at random instead, each
// rejected candidate redrawn, so seeded synthetic boxes of any size can be
// made quickly.  Pure host code, no CUDA.
#include <cmath>
#include <cstdint>
#include <vector>

namespace {

// splitmix64 (seeding) and xoshiro256** (Blackman & Vigna, 2018), restated
// from their published descriptions.
uint64_t splitmix64(uint64_t& s) {
  uint64_t z = (s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

struct Xoshiro {
  uint64_t s[4];
  explicit Xoshiro(uint64_t seed) {
    for (auto& v : s) v = splitmix64(seed);
  }
  static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
  uint64_t next() {
    const uint64_t r = rotl(s[1] * 5, 7) * 9;
    const uint64_t t = s[1] << 17;
    s[2] ^= s[0];
    s[3] ^= s[1];
    s[1] ^= s[2];
    s[0] ^= s[3];
    s[2] ^= t;
    s[3] = rotl(s[3], 45);
    return r;
  }
  double uniform() { return (double)(next() >> 11) * 0x1.0p-53; }
};

}  // namespace

extern "C" int mcgpu_build_centres(int n, double L, double dmin, uint64_t seed, double* out) {
  if (n < 0 || !(L > 0) || !(dmin >= 0) || (n > 0 && !out)) return 1;
  if (n == 0) return 0;
  int nc = dmin > 0 ? (int)std::floor(L / dmin) : 1;
  if (nc < 3) nc = 1;
  if (nc > 512) nc = 512;
  const double cw = L / nc;
  std::vector<std::vector<int>> cells((size_t)nc * nc * nc);
  Xoshiro rng(seed);
  const double d2 = dmin * dmin;
  const long long max_tries = 2000LL * n + 100000;
  long long tries = 0;
  int k = 0;
  while (k < n) {
    if (++tries > max_tries) return 2;
    const double p[3] = {rng.uniform() * L, rng.uniform() * L, rng.uniform() * L};
    int c[3];
    for (int d = 0; d < 3; d++) {
      c[d] = (int)(p[d] / cw);
      if (c[d] >= nc) c[d] = nc - 1;
      if (nc < 3) c[d] = 0;  // with < 3 cells per edge one cell covers the box
    }
    bool ok = true;
    const int span = nc >= 3 ? 1 : 0;
    for (int a = -span; a <= span && ok; a++)
      for (int b = -span; b <= span && ok; b++)
        for (int e = -span; e <= span && ok; e++) {
          const int ca = (c[0] + a + nc) % nc, cb = (c[1] + b + nc) % nc, ce = (c[2] + e + nc) % nc;
          const std::vector<int>& cell = cells[((size_t)ca * nc + cb) * nc + ce];
          for (int j : cell) {
            double r2 = 0;
            for (int d = 0; d < 3; d++) {
              double dx = out[3 * j + d] - p[d];
              dx -= L * std::nearbyint(dx / L);
              r2 += dx * dx;
            }
            if (r2 < d2) {
              ok = false;
              break;
            }
          }
        }
    if (!ok) continue;
    cells[((size_t)c[0] * nc + c[1]) * nc + c[2]].push_back(k);
    for (int d = 0; d < 3; d++) out[3 * k + d] = p[d];
    k++;
  }
  return 0;
}
