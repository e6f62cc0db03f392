// glibc's rand() as a stand-alone generator.
//
// The reference picks each BVH node's split axis with rand() % 3
// (src/ray-tracing/Bvh.h:42-45, called once per popped node at :160) and
// never seeds, so its tree depends on glibc's default generator. The GPU
// builder needs the same axis sequence; this file produces it from the
// published description of glibc's TYPE_3 additive feedback generator
// (degree 31, separation 3; see P. Selinger, "The GLIBC pseudo-random number
// generator", 2007):
//   r[0] = seed (0 -> 1); r[i] = 16807 * r[i-1] mod (2^31 - 1) for i < 31
//   (Schrage's method on a signed 32-bit word, as glibc computes it);
//   r[i] = r[i-31] for 31 <= i < 34;
//   r[i] = r[i-31] + r[i-3] (mod 2^32) for i >= 34;
//   the k-th rand() is r[k + 344] >> 1.
// The tests pin it against the C library's rand().
#include <cstdint>
#include <vector>

#include "rt_internal.h"

namespace rtgb {
namespace {

struct GlibcRand {
  uint32_t ring[34];
  uint64_t i;  // index of the next r[] to produce
  explicit GlibcRand(uint32_t seed) {
    if (seed == 0) seed = 1;
    // The seed is carried as a signed 32-bit word, so seeds >= 2^31 start
    // negative; Schrage's step then runs on 64-bit intermediates.
    int32_t word = (int32_t)seed;
    uint32_t r[34];
    r[0] = seed;
    for (int k = 1; k < 31; k++) {
      int64_t hi = (int64_t)word / 127773, lo = (int64_t)word % 127773;
      word = (int32_t)(16807 * lo - 2836 * hi);
      if (word < 0) word += 2147483647;
      r[k] = (uint32_t)word;
    }
    for (int k = 31; k < 34; k++) r[k] = r[k - 31];
    for (int k = 0; k < 34; k++) ring[k] = r[k];
    i = 34;
    for (int k = 0; k < 310; k++) step();
  }
  // Produces r[i] and advances; ring holds r[i-34 .. i-1] modulo 34.
  uint32_t step() {
    uint32_t v = ring[(i - 31) % 34] + ring[(i - 3) % 34];
    ring[i % 34] = v;
    i++;
    return v;
  }
  int32_t next() { return (int32_t)(step() >> 1); }
};

}  // namespace

void glibc_rand_values(uint32_t seed, uint64_t count, int32_t *out) {
  GlibcRand g(seed);
  for (uint64_t k = 0; k < count; k++) out[k] = g.next();
}

void glibc_rand_axes(uint32_t seed, uint64_t count, uint8_t *out_mod3) {
  GlibcRand g(seed);
  for (uint64_t k = 0; k < count; k++) out_mod3[k] = (uint8_t)(g.next() % 3);
}

}  // namespace rtgb

extern "C" void rtgbGlibcRand(uint32_t seed, uint64_t count, int32_t *out) {
  rtgb::glibc_rand_values(seed, count, out);
}
