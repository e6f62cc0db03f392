// Test harness: the GPU builder's std::sort replay (sort_emul.cuh, compiled
// here as host code) against libstdc++'s own std::sort and depth-limited
// introsort on random inputs with many ties. Prints "ok <cases>" or the
// first mismatch and exits non-zero.
#include <algorithm>
#include <cstdio>
#include <random>
#include <vector>

#include "sort_emul.cuh"

struct Item {
  float k;
  uint32_t v;
};

int main() {
  std::mt19937 rng(12345);
  int cases = 0;
  for (int t = 0; t < 30000; t++) {
    int n = (t % 9 == 0) ? (int)(rng() % 6000) : (int)(rng() % 300);
    int distinct = 1 + (int)(rng() % (t % 3 == 0 ? 5 : 2000));
    std::vector<float> k(n);
    std::vector<uint32_t> v(n);
    for (int i = 0; i < n; i++) {
      k[i] = (float)(rng() % distinct) * 0.25f - 3.0f;
      v[i] = i;
    }
    if (t % 11 == 0) std::sort(k.begin(), k.end());
    if (t % 13 == 0) std::sort(k.rbegin(), k.rend());
    std::vector<Item> ref(n);
    for (int i = 0; i < n; i++) ref[i] = {k[i], v[i]};
    auto cmp = [](const Item &a, const Item &b) { return a.k < b.k; };
    int depth = (t % 5 == 0) ? (int)(rng() % 4) : -1;
    if (depth < 0) {
      std::sort(ref.begin(), ref.end(), cmp);
      rtgb::sortemu::seq_sort<64>(k.data(), v.data(), n);
    } else if (n > 1) {
      std::__introsort_loop(ref.begin(), ref.end(), (long)depth, __gnu_cxx::__ops::__iter_comp_iter(cmp));
      std::__final_insertion_sort(ref.begin(), ref.end(), __gnu_cxx::__ops::__iter_comp_iter(cmp));
      rtgb::sortemu::seq_sort_from<64>(k.data(), v.data(), n, depth);
    }
    for (int i = 0; i < n; i++) {
      if (ref[i].v != v[i]) {
        std::printf("mismatch case %d n=%d depth=%d at %d\n", t, n, depth, i);
        return 1;
      }
    }
    cases++;
  }
  std::printf("ok %d\n", cases);
  return 0;
}
