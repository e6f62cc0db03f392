// The permutation std::sort produces, reproduced step for step.
//
// The reference orders each BVH node's triangles with std::sort on a key
// that ties often (Bvh.h:166 via boxCompare, Bvh.h:116-122), and std::sort
// is not stable, so which of two equal keys lands left of the median — and
// the order both children inherit — is decided by libstdc++'s introsort. To
// build the reference's node array bit-exact, the GPU builder replays that
// algorithm as documented for libstdc++ (GCC 13):
//   sort(first,last):    if n > 1: introsort_loop(first, last, 2*floor(log2 n));
//                        final_insertion_sort(first, last)
//   introsort_loop:      while (last-first > 16) {
//                          if depth == 0: heap sort [first,last) and return
//                          --depth; cut = unguarded_partition_pivot(first,last)
//                          introsort_loop(cut, last, depth); last = cut }
//   partition_pivot:     move the median of (first+1, mid, last-1) to first,
//                        then Hoare-partition [first+1,last) around *first with
//                        unguarded scans (stop at !(x < pivot) from the left
//                        and at !(pivot < x) from the right), swapping pairs
//                        until the scans cross; the cut is the left scan's stop.
//   heap sort:           make_heap + sort_heap with the "hole" sift-down that
//                        follows the larger child and then sifts the value up.
//   final insertion:     a stable insertion sort of the whole range.
// The sequential functions here serve tiny ranges and the heap-sort fallback;
// bvh_build.cu reproduces the partition in parallel (same swaps, same cut).
// Every comparison is the strict `key[a] < key[b]` of the reference's
// comparator; keys are finite (the upload rejects non-finite vertices).
#pragma once
#include <stdint.h>

#ifdef __CUDACC__
#define RTGB_HD __host__ __device__ __forceinline__
#else
#define RTGB_HD inline
#endif

namespace rtgb {
namespace sortemu {

RTGB_HD void swap_at(float *k, uint32_t *v, long a, long b) {
  float tk = k[a];
  k[a] = k[b];
  k[b] = tk;
  uint32_t tv = v[a];
  v[a] = v[b];
  v[b] = tv;
}

RTGB_HD int floor_log2(unsigned long n) {
  int r = 0;
  while (n > 1) {
    n >>= 1;
    r++;
  }
  return r;
}

// Sift the value (vk, vv) up from `hole` towards `top`.
RTGB_HD void push_heap(float *k, uint32_t *v, long hole, long top, float vk, uint32_t vv) {
  long parent = (hole - 1) / 2;
  while (hole > top && k[parent] < vk) {
    k[hole] = k[parent];
    v[hole] = v[parent];
    hole = parent;
    parent = (hole - 1) / 2;
  }
  k[hole] = vk;
  v[hole] = vv;
}

// Move the hole at `hole` down to a leaf along the larger child, then sift
// (vk, vv) up from there.
RTGB_HD void adjust_heap(float *k, uint32_t *v, long hole, long len, float vk, uint32_t vv) {
  const long top = hole;
  long child = hole;
  while (child < (len - 1) / 2) {
    child = 2 * (child + 1);
    if (k[child] < k[child - 1]) child--;
    k[hole] = k[child];
    v[hole] = v[child];
    hole = child;
  }
  if ((len & 1) == 0 && child == (len - 2) / 2) {
    child = 2 * (child + 1);
    k[hole] = k[child - 1];
    v[hole] = v[child - 1];
    hole = child - 1;
  }
  push_heap(k, v, hole, top, vk, vv);
}

// make_heap followed by sort_heap on [0, n).
RTGB_HD void heap_sort(float *k, uint32_t *v, long n) {
  if (n < 2) return;
  for (long parent = (n - 2) / 2;; parent--) {
    adjust_heap(k, v, parent, n, k[parent], v[parent]);
    if (parent == 0) break;
  }
  for (long last = n - 1; last > 0; last--) {
    float vk = k[last];
    uint32_t vv = v[last];
    k[last] = k[0];
    v[last] = v[0];
    adjust_heap(k, v, 0, last, vk, vv);
  }
}

// Stable insertion sort of [0, n).
RTGB_HD void insertion_sort(float *k, uint32_t *v, long n) {
  for (long i = 1; i < n; i++) {
    float vk = k[i];
    uint32_t vv = v[i];
    long j = i;
    while (j > 0 && vk < k[j - 1]) {
      k[j] = k[j - 1];
      v[j] = v[j - 1];
      j--;
    }
    k[j] = vk;
    v[j] = vv;
  }
}

// Median of (a, b, c) moved to `result` (all offsets into k/v).
RTGB_HD void median_to_first(float *k, uint32_t *v, long result, long a, long b, long c) {
  if (k[a] < k[b]) {
    if (k[b] < k[c])
      swap_at(k, v, result, b);
    else if (k[a] < k[c])
      swap_at(k, v, result, c);
    else
      swap_at(k, v, result, a);
  } else if (k[a] < k[c]) {
    swap_at(k, v, result, a);
  } else if (k[b] < k[c]) {
    swap_at(k, v, result, c);
  } else {
    swap_at(k, v, result, b);
  }
}

// Sequential unguarded partition of [first+1, last) around k[first]
// (after median_to_first); returns the cut.
RTGB_HD long partition_pivot(float *k, uint32_t *v, long first, long last) {
  long mid = first + (last - first) / 2;
  median_to_first(k, v, first, first + 1, mid, last - 1);
  const float pk = k[first];
  long lo = first + 1, hi = last;
  for (;;) {
    while (k[lo] < pk) lo++;
    hi--;
    while (pk < k[hi]) hi--;
    if (!(lo < hi)) return lo;
    swap_at(k, v, lo, hi);
    lo++;
  }
}

// Full std::sort replay of [0, n) with an explicit range stack (ranges are
// disjoint, so the order they are processed in does not change the result).
template <int MAXSTACK>
RTGB_HD void seq_sort_from(float *k, uint32_t *v, long n, int depth) {
  long sf[MAXSTACK], sl[MAXSTACK];
  int sd[MAXSTACK];
  int sp = 0;
  sf[sp] = 0;
  sl[sp] = n;
  sd[sp] = depth;
  sp++;
  while (sp > 0) {
    sp--;
    long f = sf[sp], l = sl[sp];
    int d = sd[sp];
    while (l - f > 16) {
      if (d == 0) {
        heap_sort(k + f, v + f, l - f);
        break;
      }
      d--;
      long cut = partition_pivot(k, v, f, l);
      if (sp < MAXSTACK) {
        sf[sp] = cut;
        sl[sp] = l;
        sd[sp] = d;
        sp++;
      }
      l = cut;
    }
  }
  insertion_sort(k, v, n);
}

template <int MAXSTACK>
RTGB_HD void seq_sort(float *k, uint32_t *v, long n) {
  if (n > 1) seq_sort_from<MAXSTACK>(k, v, n, 2 * floor_log2((unsigned long)n));
}

}  // namespace sortemu
}  // namespace rtgb
