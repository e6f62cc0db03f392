// GPU BVH build, node-for-node identical to Bvh::createBvh
// (src/ray-tracing/Bvh.h:141-209).
//
// What the reference does, and what decides each output word:
//   * Topology. A node with n triangles gets n/2 on the left and the rest on
//     the right (Bvh.h:175-197); the DFS stack pops the right child first and
//     the creation counter names children 2k+1 / 2k+2 when the k-th inner
//     node is popped (Bvh.h:178-192). So indices, child links and the order
//     in which nodes draw rand() depend on n alone; the host derives them
//     in O(n) (pop rank of the right child = parent + 1, of the left child =
//     parent + 2*|right| ; inner rank = pop rank - leaves popped before).
//   * Axis. rand() % 3 once per popped node, leaves included (Bvh.h:160);
//     the host supplies glibc's sequence (glibc_rand.cpp).
//   * Which triangles a child receives, and in what order, is the sorted
//     order of its parent's triangles under std::sort (Bvh.h:166) with the
//     key min(v0,v1,v2)[axis] - 1e-4 (Bvh.h:94-98,116-122). Ties are common,
//     so the sort is replayed exactly (sort_emul.cuh).
//   * Boxes are unions of padded triangle boxes (Bvh.h:94-114); min/max are
//     order-free on finite values, so they are computed bottom-up at the end.
//
// GPU organisation. All triangles live in one array `idx`; a node owns the
// slice [off, off+n), and sorting a node in place leaves its children's
// slices in their input order. Nodes of one tree level are independent, so
// the build runs level by level:
//   1. k_keys    — every element's key for its node's axis.
//   2. k_sort_big — one 1024-thread CTA per node larger than kWarpMax:
//                  introsort partitions done cooperatively (the swap pairs of
//                  an unguarded Hoare partition are the i-th "!(x < p)" from
//                  the left and the i-th "!(p < x)" from the right, found with
//                  block scans; the cut is min(P[K+1], Q[K]) for the largest
//                  K with P[K] < Q[K]); sub-ranges of <= kWarpMax go to a queue.
//   3. k_sort_warps — a persistent grid of warps drains the queue: warp-wide
//                  partitions (ballot/popc scans) down to 16 elements, then a
//                  rank-based stable sort of each <= 16 block (what the final
//                  insertion sort does to it), heap sort where the depth
//                  limit runs out.
// Then leaves are written and inner boxes reduced bottom-up.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <vector>

#include "rt_internal.h"
#include "sort_emul.cuh"

namespace rtgb {
namespace {

constexpr uint32_t kWarpMax = 8192;  // ranges up to this size are finished by one warp
constexpr int kBigThreads = 1024;
constexpr int kWarpStack = 64;

struct Seg {
  uint32_t off, n, node, kchild;  // children are nodes 2*kchild+1 (left), 2*kchild+2
  uint32_t axis, depth;           // split axis; introsort depth limit 2*floor(log2 n)
};
struct Leaf {
  uint32_t node, off;
};
struct Range {
  uint32_t f, l, d;
};

__device__ __forceinline__ float tri_key(const rt_triangle &t, int axis) {
  float a = t.v0[axis], b = t.v1[axis], c = t.v2[axis];
  float m = (b < a) ? b : a;
  m = (c < m) ? c : m;
  return __fsub_rn(m, 0.0001f);
}

__global__ void k_iota(uint32_t *idx, uint32_t n) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) idx[i] = i;
}

// Test hook of the build's error word: records `bits` as a sort kernel
// would on an overflow, so a test can check that an error raised at any
// level survives to the end of the build.
__global__ void k_flag_error(uint32_t *err, uint32_t bits) { atomicOr(err, bits); }

// Every vertex coordinate must be finite: the sort replay orders keys with
// IEEE `<`, which a NaN key breaks, and node boxes are min/max unions. Any
// non-finite coordinate sets `bits` in the error word.
__global__ void k_check_finite(const rt_triangle *__restrict__ tris, uint32_t n, uint32_t *err, uint32_t bits) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const rt_triangle t = tris[i];
  bool ok = true;
  for (int k = 0; k < 3; k++) ok = ok && isfinite(t.v0[k]) && isfinite(t.v1[k]) && isfinite(t.v2[k]);
  if (!ok) atomicOr(err, bits);
}

// Key of every element that belongs to a node of this level with n >= 2.
__global__ void k_keys(const Seg *__restrict__ segs, uint32_t nseg, const rt_triangle *__restrict__ tris,
                       const uint32_t *__restrict__ idx, float *__restrict__ key, uint32_t n) {
  uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  uint32_t lo = 0, hi = nseg;  // last segment with off <= e
  while (hi - lo > 1) {
    uint32_t m = (lo + hi) >> 1;
    if (segs[m].off <= e) lo = m; else hi = m;
  }
  const Seg s = segs[lo];
  if (e < s.off || e >= s.off + s.n) return;
  key[e] = tri_key(tris[idx[e]], (int)s.axis);
}

__global__ void k_enqueue(const Seg *__restrict__ segs, uint32_t nseg, Range *queue, uint32_t *qcount) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nseg) return;
  const Seg s = segs[i];
  if (s.n > kWarpMax) return;
  uint32_t slot = atomicAdd(qcount, 1u);
  queue[slot] = Range{s.off, s.off + s.n, s.depth};
}

// ------------------------------------------------------------ CTA partition
__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v, uint32_t *warp_tot, uint32_t &total) {
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= (uint32_t)o) x += y;
  }
  if (lane == 31) warp_tot[warp] = x;
  __syncthreads();
  if (warp == 0) {
    uint32_t w = warp_tot[lane];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= (uint32_t)o) w += y;
    }
    warp_tot[lane] = w;
  }
  __syncthreads();
  uint32_t excl = x - v + (warp > 0 ? warp_tot[warp - 1] : 0u);
  total = warp_tot[31];
  __syncthreads();
  return excl;
}

struct BigShared {
  uint32_t warp_tot[32];
  uint32_t sf[kWarpStack], sl[kWarpStack], sd[kWarpStack];
  uint32_t sp;
  uint32_t cur_f, cur_l, cur_d;
  uint32_t K, cut;
};

__device__ uint32_t cta_partition(float *key, uint32_t *idx, uint32_t f, uint32_t l, uint32_t *P, uint32_t *Q,
                                  BigShared &sh) {
  if (threadIdx.x == 0) {
    uint32_t mid = f + (l - f) / 2;
    sortemu::median_to_first(key, idx, f, f + 1, mid, l - 1);
  }
  __syncthreads();
  const float pk = key[f];
  // Totals of "!(x < p)" (ge) and "!(p < x)" (le) over [f+1, l), packed
  // 16/16 per chunk of kBigThreads.
  uint32_t GE = 0, LE = 0;
  for (uint32_t base = f + 1; base < l; base += kBigThreads) {
    uint32_t i = base + threadIdx.x;
    uint32_t packed = 0;
    if (i < l) {
      float k = key[i];
      packed = (!(k < pk) ? 1u : 0u) | (!(pk < k) ? 0x10000u : 0u);
    }
    uint32_t tot;
    block_excl_scan(packed, sh.warp_tot, tot);
    GE += tot & 0xffffu;
    LE += tot >> 16;
  }
  // Rank lists: P[f + j] = j-th ge position from the left,
  // Q[f + j] = j-th le position from the right.
  uint32_t cg = 0, cl = 0;
  for (uint32_t base = f + 1; base < l; base += kBigThreads) {
    uint32_t i = base + threadIdx.x;
    uint32_t packed = 0;
    if (i < l) {
      float k = key[i];
      packed = (!(k < pk) ? 1u : 0u) | (!(pk < k) ? 0x10000u : 0u);
    }
    uint32_t tot;
    uint32_t ex = block_excl_scan(packed, sh.warp_tot, tot);
    if (packed & 1u) P[f + cg + (ex & 0xffffu)] = i;
    if (packed & 0x10000u) Q[f + (LE - 1u - (cl + (ex >> 16)))] = i;
    cg += tot & 0xffffu;
    cl += tot >> 16;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t lo = 0, hi = GE < LE ? GE : LE;
    while (lo < hi) {
      uint32_t m = (lo + hi + 1) >> 1;
      if (P[f + m - 1] < Q[f + m - 1]) lo = m; else hi = m - 1;
    }
    uint32_t cut = lo < GE ? P[f + lo] : 0xffffffffu;
    if (lo >= 1 && Q[f + lo - 1] < cut) cut = Q[f + lo - 1];
    sh.K = lo;
    sh.cut = cut;
  }
  __syncthreads();
  const uint32_t K = sh.K;
  for (uint32_t j = threadIdx.x; j < K; j += kBigThreads) {
    uint32_t a = P[f + j], b = Q[f + j];
    float ka = key[a], kb = key[b];
    uint32_t va = idx[a], vb = idx[b];
    key[a] = kb;
    idx[a] = vb;
    key[b] = ka;
    idx[b] = va;
  }
  __syncthreads();
  return sh.cut;
}

__global__ void __launch_bounds__(kBigThreads) k_sort_big(const Seg *__restrict__ segs, float *key, uint32_t *idx,
                                                          uint32_t *P, uint32_t *Q, Range *queue,
                                                          uint32_t *qcount, uint32_t *err) {
  __shared__ BigShared sh;
  const Seg s = segs[blockIdx.x];
  if (s.n <= kWarpMax) return;  // queued by k_enqueue
  if (threadIdx.x == 0) {
    sh.sf[0] = s.off;
    sh.sl[0] = s.off + s.n;
    sh.sd[0] = s.depth;
    sh.sp = 1;
  }
  __syncthreads();
  for (;;) {
    if (threadIdx.x == 0) {
      if (sh.sp == 0) {
        sh.cur_l = 0;
        sh.cur_f = 0;
      } else {
        sh.sp--;
        sh.cur_f = sh.sf[sh.sp];
        sh.cur_l = sh.sl[sh.sp];
        sh.cur_d = sh.sd[sh.sp];
      }
    }
    __syncthreads();
    const uint32_t f = sh.cur_f, l = sh.cur_l, d = sh.cur_d;
    if (l == 0) break;
    if (l - f <= kWarpMax) {
      if (threadIdx.x == 0) {
        uint32_t slot = atomicAdd(qcount, 1u);
        queue[slot] = Range{f, l, d};
      }
      __syncthreads();
      continue;
    }
    if (d == 0) {
      if (threadIdx.x == 0) sortemu::heap_sort(key + f, idx + f, (long)(l - f));
      __syncthreads();
      continue;
    }
    uint32_t cut = cta_partition(key, idx, f, l, P, Q, sh);
    if (cut <= f || cut >= l) {
      // Cannot happen for finite keys (the median-of-three guards both
      // scans); keep the ranges in bounds regardless.
      if (threadIdx.x == 0) {
        atomicOr(err, KERR_BAD_INDEX);
        sortemu::heap_sort(key + f, idx + f, (long)(l - f));
      }
      __syncthreads();
      continue;
    }
    if (threadIdx.x == 0) {
      if (sh.sp + 2 > kWarpStack) {
        atomicOr(err, KERR_STACK_OVERFLOW);
        sh.sp = 0;
      } else {
        sh.sf[sh.sp] = cut;
        sh.sl[sh.sp] = l;
        sh.sd[sh.sp] = d - 1;
        sh.sp++;
        sh.sf[sh.sp] = f;
        sh.sl[sh.sp] = cut;
        sh.sd[sh.sp] = d - 1;
        sh.sp++;
      }
    }
    __syncthreads();
  }
}

// ------------------------------------------------------------ warp ranges
__device__ uint32_t warp_partition(float *key, uint32_t *idx, uint32_t f, uint32_t l, uint32_t *P, uint32_t *Q,
                                   uint32_t lane) {
  if (lane == 0) {
    uint32_t mid = f + (l - f) / 2;
    sortemu::median_to_first(key, idx, f, f + 1, mid, l - 1);
  }
  __syncwarp();
  const float pk = key[f];
  const uint32_t lt = (1u << lane) - 1u;
  uint32_t GE = 0, LE = 0;
  for (uint32_t base = f + 1; base < l; base += 32) {
    uint32_t i = base + lane;
    bool ge = false, le = false;
    if (i < l) {
      float k = key[i];
      ge = !(k < pk);
      le = !(pk < k);
    }
    GE += __popc(__ballot_sync(0xffffffffu, ge));
    LE += __popc(__ballot_sync(0xffffffffu, le));
  }
  uint32_t cg = 0, cl = 0;
  for (uint32_t base = f + 1; base < l; base += 32) {
    uint32_t i = base + lane;
    bool ge = false, le = false;
    if (i < l) {
      float k = key[i];
      ge = !(k < pk);
      le = !(pk < k);
    }
    uint32_t bg = __ballot_sync(0xffffffffu, ge), bl = __ballot_sync(0xffffffffu, le);
    if (ge) P[f + cg + __popc(bg & lt)] = i;
    if (le) Q[f + (LE - 1u - (cl + __popc(bl & lt)))] = i;
    cg += __popc(bg);
    cl += __popc(bl);
  }
  __syncwarp();
  uint32_t K = 0, cut = 0;
  if (lane == 0) {
    uint32_t lo = 0, hi = GE < LE ? GE : LE;
    while (lo < hi) {
      uint32_t m = (lo + hi + 1) >> 1;
      if (P[f + m - 1] < Q[f + m - 1]) lo = m; else hi = m - 1;
    }
    cut = lo < GE ? P[f + lo] : 0xffffffffu;
    if (lo >= 1 && Q[f + lo - 1] < cut) cut = Q[f + lo - 1];
    K = lo;
  }
  K = __shfl_sync(0xffffffffu, K, 0);
  cut = __shfl_sync(0xffffffffu, cut, 0);
  for (uint32_t j = lane; j < K; j += 32) {
    uint32_t a = P[f + j], b = Q[f + j];
    float ka = key[a], kb = key[b];
    uint32_t va = idx[a], vb = idx[b];
    key[a] = kb;
    idx[a] = vb;
    key[b] = ka;
    idx[b] = va;
  }
  __syncwarp();
  return cut;
}

// Stable sort of a block of <= 16 elements: each lane places its element at
// (#smaller keys) + (#equal keys before it).
__device__ __forceinline__ void warp_small_sort(float *key, uint32_t *idx, uint32_t f, uint32_t n, uint32_t lane) {
  bool valid = lane < n;
  float k = valid ? key[f + lane] : 0.0f;
  uint32_t v = valid ? idx[f + lane] : 0u;
  uint32_t rank = 0;
  for (uint32_t j = 0; j < n; j++) {
    float kj = __shfl_sync(0xffffffffu, k, j);
    if (kj < k || (!(k < kj) && j < lane)) rank++;
  }
  __syncwarp();
  if (valid) {
    key[f + rank] = k;
    idx[f + rank] = v;
  }
  __syncwarp();
}

__global__ void k_sort_warps(float *key, uint32_t *idx, uint32_t *P, uint32_t *Q, const Range *__restrict__ queue,
                             const uint32_t *qcount, uint32_t *qhead, uint32_t *err) {
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t count = *qcount;
  uint32_t sf[kWarpStack], sl[kWarpStack], sd[kWarpStack];
  for (;;) {
    uint32_t qi = 0;
    if (lane == 0) qi = atomicAdd(qhead, 1u);
    qi = __shfl_sync(0xffffffffu, qi, 0);
    if (qi >= count) return;
    const Range r = queue[qi];
    int sp = 0;
    sf[0] = r.f;
    sl[0] = r.l;
    sd[0] = r.d;
    sp = 1;
    while (sp > 0) {
      sp--;
      uint32_t f = sf[sp], l = sl[sp], d = sd[sp];
      uint32_t n = l - f;
      if (n <= 16) {
        if (n > 1) warp_small_sort(key, idx, f, n, lane);
        continue;
      }
      if (d == 0) {
        if (lane == 0) sortemu::heap_sort(key + f, idx + f, (long)n);
        __syncwarp();
        continue;
      }
      uint32_t cut = warp_partition(key, idx, f, l, P, Q, lane);
      if (cut <= f || cut >= l) {  // impossible for finite keys; stay in bounds
        if (lane == 0) {
          atomicOr(err, KERR_BAD_INDEX);
          sortemu::heap_sort(key + f, idx + f, (long)n);
        }
        __syncwarp();
        continue;
      }
      if (sp + 2 > kWarpStack) {
        if (lane == 0) atomicOr(err, KERR_STACK_OVERFLOW);
        return;
      }
      sf[sp] = cut;
      sl[sp] = l;
      sd[sp] = d - 1;
      sp++;
      sf[sp] = f;
      sl[sp] = cut;
      sd[sp] = d - 1;
      sp++;
    }
  }
}

// ------------------------------------------------------------ node output
__global__ void k_leaves(const Leaf *__restrict__ leaves, uint32_t nleaf, const uint32_t *__restrict__ idx,
                         const rt_triangle *__restrict__ tris, rt_bvh_node *nodes) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nleaf) return;
  const Leaf lf = leaves[i];
  uint32_t o = idx[lf.off];
  const rt_triangle t = tris[o];
  rt_bvh_node nd;
  for (int a = 0; a < 3; a++) {
    float lo = (t.v1[a] < t.v0[a]) ? t.v1[a] : t.v0[a];
    lo = (t.v2[a] < lo) ? t.v2[a] : lo;
    float hi = (t.v0[a] < t.v1[a]) ? t.v1[a] : t.v0[a];
    hi = (hi < t.v2[a]) ? t.v2[a] : hi;
    nd.min[a] = __fsub_rn(lo, 0.0001f);
    nd.max[a] = __fadd_rn(hi, 0.0001f);
  }
  nd._pad0 = 0.0f;
  nd.left = -1;
  nd.right = -1;
  nd.object = (int32_t)o;
  nd._pad1[0] = nd._pad1[1] = 0;
  nodes[lf.node] = nd;
}

__global__ void k_inner(const Seg *__restrict__ segs, uint32_t nseg, rt_bvh_node *nodes) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nseg) return;
  const Seg s = segs[i];
  uint32_t L = 2 * s.kchild + 1, R = 2 * s.kchild + 2;
  const rt_bvh_node a = nodes[L], b = nodes[R];
  rt_bvh_node nd;
  for (int k = 0; k < 3; k++) {
    nd.min[k] = (b.min[k] < a.min[k]) ? b.min[k] : a.min[k];
    nd.max[k] = (a.max[k] < b.max[k]) ? b.max[k] : a.max[k];
  }
  nd._pad0 = 0.0f;
  nd.left = (int32_t)L;
  nd.right = (int32_t)R;
  nd.object = -1;
  nd._pad1[0] = nd._pad1[1] = 0;
  nodes[s.node] = nd;
}

struct HostTopo {
  std::vector<Seg> segs;            // inner nodes, level by level, by offset
  std::vector<uint32_t> level_off;  // segs index where each level starts
  std::vector<Leaf> leaves;
  uint32_t levels = 0;
};

// O(n) replay of the reference's DFS bookkeeping, breadth first.
HostTopo host_topology(uint32_t n, const uint8_t *axes) {
  struct Item {
    uint32_t off, n, node;
    uint64_t rank, leaves_before;
  };
  HostTopo t;
  std::vector<Item> cur{Item{0, n, 0, 0, 0}}, next;
  while (!cur.empty()) {
    t.level_off.push_back((uint32_t)t.segs.size());
    t.levels++;
    next.clear();
    for (const Item &it : cur) {
      if (it.n <= 1) {
        t.leaves.push_back(Leaf{it.node, it.off});
        continue;
      }
      uint32_t k = (uint32_t)(it.rank - it.leaves_before);
      uint32_t nl = it.n / 2, nr = it.n - nl;
      Seg s;
      s.off = it.off;
      s.n = it.n;
      s.node = it.node;
      s.kchild = k;
      s.axis = axes[it.rank];
      s.depth = 2u * (uint32_t)sortemu::floor_log2(it.n);
      t.segs.push_back(s);
      next.push_back(Item{it.off, nl, 2 * k + 1, it.rank + 1 + (2ull * nr - 1), it.leaves_before + nr});
      next.push_back(Item{it.off + nl, nr, 2 * k + 2, it.rank + 1, it.leaves_before});
    }
    cur.swap(next);
  }
  t.level_off.push_back((uint32_t)t.segs.size());
  return t;
}

#define BUILD_CHECK(x)                                                                       \
  do {                                                                                       \
    cudaError_t e_ = (x);                                                                    \
    if (e_ != cudaSuccess) {                                                                 \
      std::snprintf(errbuf, errlen, "bvh build: %s (%s:%d)", cudaGetErrorString(e_), __FILE__, \
                    __LINE__);                                                               \
      status = RT_ERR_CUDA;                                                                  \
      goto done;                                                                             \
    }                                                                                        \
  } while (0)

}  // namespace

rt_status gpu_build_bvh(const rt_triangle *d_tris, uint32_t n, const uint8_t *h_axes, rt_bvh_node *d_nodes,
                        cudaStream_t st, float *ms_out, uint32_t *depth_out, char *errbuf, size_t errlen,
                        int test_error_level) {
  rt_status status = RT_SUCCESS;
  HostTopo topo = host_topology(n, h_axes);
  float *key = nullptr;
  uint32_t *idx = nullptr, *P = nullptr, *Q = nullptr, *ctr = nullptr;
  Range *queue = nullptr;
  Seg *dsegs = nullptr;
  Leaf *dleaves = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int sms = 0, dev = 0;
  const uint32_t nseg_all = (uint32_t)topo.segs.size();
  BUILD_CHECK(cudaGetDevice(&dev));
  BUILD_CHECK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  BUILD_CHECK(cudaEventCreate(&e0));
  BUILD_CHECK(cudaEventCreate(&e1));
  BUILD_CHECK(cudaMallocAsync((void **)&key, sizeof(float) * n, st));
  BUILD_CHECK(cudaMallocAsync((void **)&idx, sizeof(uint32_t) * n, st));
  BUILD_CHECK(cudaMallocAsync((void **)&P, sizeof(uint32_t) * n, st));
  BUILD_CHECK(cudaMallocAsync((void **)&Q, sizeof(uint32_t) * n, st));
  BUILD_CHECK(cudaMallocAsync((void **)&queue, sizeof(Range) * n, st));
  BUILD_CHECK(cudaMallocAsync((void **)&ctr, sizeof(uint32_t) * 4, st));
  BUILD_CHECK(cudaMallocAsync((void **)&dsegs, sizeof(Seg) * (nseg_all ? nseg_all : 1), st));
  BUILD_CHECK(cudaMallocAsync((void **)&dleaves, sizeof(Leaf) * topo.leaves.size(), st));
  if (nseg_all)
    BUILD_CHECK(cudaMemcpyAsync(dsegs, topo.segs.data(), sizeof(Seg) * nseg_all, cudaMemcpyHostToDevice, st));
  BUILD_CHECK(cudaMemcpyAsync(dleaves, topo.leaves.data(), sizeof(Leaf) * topo.leaves.size(),
                              cudaMemcpyHostToDevice, st));
  BUILD_CHECK(cudaEventRecord(e0, st));
  // ctr: [0] queue count, [1] queue head (both per level), [2] error bits
  // (kept across levels), [3] unused.
  BUILD_CHECK(cudaMemsetAsync(ctr, 0, sizeof(uint32_t) * 4, st));
  k_iota<<<(n + 255) / 256, 256, 0, st>>>(idx, n);
  for (uint32_t L = 0; L < topo.levels; L++) {
    uint32_t s0 = topo.level_off[L], s1 = topo.level_off[L + 1];
    uint32_t ns = s1 - s0;
    if (ns == 0) continue;
    const Seg *ls = dsegs + s0;
    BUILD_CHECK(cudaMemsetAsync(ctr, 0, sizeof(uint32_t) * 2, st));
    k_keys<<<(n + 255) / 256, 256, 0, st>>>(ls, ns, d_tris, idx, key, n);
    k_enqueue<<<(ns + 255) / 256, 256, 0, st>>>(ls, ns, queue, ctr);
    // Inner nodes of one level have sizes floor or ceil of n / 2^L.
    uint32_t maxn = std::max(topo.segs[s0].n, topo.segs[s1 - 1].n);
    for (uint32_t j = s0; j < s1 && j < s0 + 2; j++) maxn = std::max(maxn, topo.segs[j].n);
    if (maxn > kWarpMax) {
      k_sort_big<<<ns, kBigThreads, 0, st>>>(ls, key, idx, P, Q, queue, ctr, ctr + 2);
    }
    uint32_t grid = (uint32_t)sms * 8u;
    k_sort_warps<<<grid, 256, 0, st>>>(key, idx, P, Q, queue, ctr, ctr + 1, ctr + 2);
    if ((int)L == test_error_level) k_flag_error<<<1, 1, 0, st>>>(ctr + 2, KERR_STACK_OVERFLOW);
    BUILD_CHECK(cudaGetLastError());
  }
  k_leaves<<<((uint32_t)topo.leaves.size() + 255) / 256, 256, 0, st>>>(dleaves, (uint32_t)topo.leaves.size(),
                                                                       idx, d_tris, d_nodes);
  for (int L = (int)topo.levels - 1; L >= 0; L--) {
    uint32_t s0 = topo.level_off[L], s1 = topo.level_off[L + 1];
    if (s1 > s0) k_inner<<<(s1 - s0 + 255) / 256, 256, 0, st>>>(dsegs + s0, s1 - s0, d_nodes);
  }
  BUILD_CHECK(cudaGetLastError());
  BUILD_CHECK(cudaEventRecord(e1, st));
  {
    uint32_t flags[4] = {0, 0, 0, 0};
    BUILD_CHECK(cudaMemcpyAsync(flags, ctr, sizeof(flags), cudaMemcpyDeviceToHost, st));
    BUILD_CHECK(cudaStreamSynchronize(st));
    if (flags[2] != 0) {
      std::snprintf(errbuf, errlen, "bvh build: internal sort error (bits 0x%x)", flags[2]);
      status = RT_ERR_INTERNAL;
    }
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms_out) *ms_out = ms;
    if (depth_out) *depth_out = topo.levels;
  }
done:
  cudaFreeAsync(key, st);
  cudaFreeAsync(idx, st);
  cudaFreeAsync(P, st);
  cudaFreeAsync(Q, st);
  cudaFreeAsync(queue, st);
  cudaFreeAsync(ctr, st);
  cudaFreeAsync(dsegs, st);
  cudaFreeAsync(dleaves, st);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  return status;
}

}  // namespace rtgb

// ---------------------------------------------------------------------------
// Allocation-free build: rtBuildBvhNoAlloc.
//
// For callers that cannot allocate device memory, the same kernels run on a
// fixed scratch area that is part of the library image: a file-scope
// __device__ array sized for kNoAllocMaxTriangles triangles (about 3.9 MB,
// held by every GPU that loads the library until the process exits). The
// host-side bookkeeping uses static buffers as well, so a call performs no
// allocation of any kind. All calls share both areas: calls must not
// overlap (they are serialised on the host by a mutex and each call waits
// for its own GPU work before returning; calls issued by other means on the
// same device while one is running would race on the shared array).
#include <mutex>

namespace rtgb {
namespace {

constexpr uint32_t kNoAllocMaxTriangles = 65536;
constexpr size_t kNaAlign(size_t x) { return (x + 255) & ~size_t(255); }
constexpr size_t kNaKey = 0;
constexpr size_t kNaIdx = kNaKey + kNaAlign(4ull * kNoAllocMaxTriangles);
constexpr size_t kNaP = kNaIdx + kNaAlign(4ull * kNoAllocMaxTriangles);
constexpr size_t kNaQ = kNaP + kNaAlign(4ull * kNoAllocMaxTriangles);
constexpr size_t kNaQueue = kNaQ + kNaAlign(4ull * kNoAllocMaxTriangles);
constexpr size_t kNaSegs = kNaQueue + kNaAlign(sizeof(Range) * kNoAllocMaxTriangles);
constexpr size_t kNaLeaves = kNaSegs + kNaAlign(sizeof(Seg) * kNoAllocMaxTriangles);
constexpr size_t kNaCtr = kNaLeaves + kNaAlign(sizeof(Leaf) * kNoAllocMaxTriangles);
constexpr size_t kNaBytes = kNaCtr + 256;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNaBytes];

struct NaItem {
  uint32_t off, n, node;
  uint64_t rank, leaves_before;
};
struct NaHost {
  uint8_t axes[2 * kNoAllocMaxTriangles];
  Seg segs[kNoAllocMaxTriangles];
  Leaf leaves[kNoAllocMaxTriangles];
  NaItem cur[kNoAllocMaxTriangles], next[kNoAllocMaxTriangles];
  uint32_t level_off[72];
  uint32_t levels, nsegs, nleaves;
  uint32_t flags[4];
};
static NaHost g_na_host;
static std::mutex g_na_mu;
constexpr int kNaMaxDevices = 64;
static unsigned char *g_na_dev[kNaMaxDevices];  // device address of the scratch array, per device

// The topology replay of host_topology() written into the static buffers.
void na_topology(uint32_t n, NaHost &h) {
  uint32_t ncur = 1, nnext = 0;
  h.cur[0] = NaItem{0, n, 0, 0, 0};
  h.levels = 0;
  h.nsegs = 0;
  h.nleaves = 0;
  while (ncur) {
    h.level_off[h.levels++] = h.nsegs;
    nnext = 0;
    for (uint32_t i = 0; i < ncur; i++) {
      const NaItem it = h.cur[i];
      if (it.n <= 1) {
        h.leaves[h.nleaves++] = Leaf{it.node, it.off};
        continue;
      }
      uint32_t k = (uint32_t)(it.rank - it.leaves_before);
      uint32_t nl = it.n / 2, nr = it.n - nl;
      Seg s;
      s.off = it.off;
      s.n = it.n;
      s.node = it.node;
      s.kchild = k;
      s.axis = h.axes[it.rank];
      s.depth = 2u * (uint32_t)sortemu::floor_log2(it.n);
      h.segs[h.nsegs++] = s;
      h.next[nnext++] = NaItem{it.off, nl, 2 * k + 1, it.rank + 1 + (2ull * nr - 1), it.leaves_before + nr};
      h.next[nnext++] = NaItem{it.off + nl, nr, 2 * k + 2, it.rank + 1, it.leaves_before};
    }
    for (uint32_t i = 0; i < nnext; i++) h.cur[i] = h.next[i];
    ncur = nnext;
  }
  h.level_off[h.levels] = h.nsegs;
}

}  // namespace
}  // namespace rtgb

extern "C" rt_status rtBuildBvhNoAlloc(const rt_triangle *d_triangles, uint32_t n, uint32_t bvh_seed,
                                       rt_bvh_node *d_nodes, void *stream) {
  using namespace rtgb;
  if (!d_triangles || !d_nodes || n == 0 || n > kNoAllocMaxTriangles) return RT_ERR_INVALID_ARGUMENT;
  if ((uintptr_t)d_triangles % 16 || (uintptr_t)d_nodes % 16) return RT_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> guard(g_na_mu);
  cudaStream_t st = (cudaStream_t)stream;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kNaMaxDevices) return RT_ERR_CUDA;
  if (!g_na_dev[dev]) {
    // Once per device, with that device current: host code cannot use the
    // array's name as a device address, so look the address up.
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return RT_ERR_CUDA;
    g_na_dev[dev] = static_cast<unsigned char *>(p);
  }
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return RT_ERR_CUDA;
  unsigned char *base = g_na_dev[dev];
  float *key = reinterpret_cast<float *>(base + kNaKey);
  uint32_t *idx = reinterpret_cast<uint32_t *>(base + kNaIdx);
  uint32_t *P = reinterpret_cast<uint32_t *>(base + kNaP);
  uint32_t *Q = reinterpret_cast<uint32_t *>(base + kNaQ);
  Range *queue = reinterpret_cast<Range *>(base + kNaQueue);
  Seg *dsegs = reinterpret_cast<Seg *>(base + kNaSegs);
  Leaf *dleaves = reinterpret_cast<Leaf *>(base + kNaLeaves);
  uint32_t *ctr = reinterpret_cast<uint32_t *>(base + kNaCtr);

  NaHost &h = g_na_host;
  glibc_rand_axes(bvh_seed, 2ull * n - 1, h.axes);
  na_topology(n, h);
  // From the first enqueue on, every return waits for the work already
  // queued on `st`: the next call (under the same lock, possibly on another
  // stream) reuses the scratch array.
  auto drain = [st](rt_status s) {
    cudaStreamSynchronize(st);
    return s;
  };
  constexpr uint32_t kNonFinite = 0x100u;
  if (h.nsegs &&
      cudaMemcpyAsync(dsegs, h.segs, sizeof(Seg) * h.nsegs, cudaMemcpyHostToDevice, st) != cudaSuccess)
    return drain(RT_ERR_CUDA);
  if (cudaMemcpyAsync(dleaves, h.leaves, sizeof(Leaf) * h.nleaves, cudaMemcpyHostToDevice, st) != cudaSuccess)
    return drain(RT_ERR_CUDA);
  // The error word survives from earlier calls: clear it.
  if (cudaMemsetAsync(ctr, 0, sizeof(uint32_t) * 4, st) != cudaSuccess) return drain(RT_ERR_CUDA);
  // Non-finite vertices are rejected before any sort runs: the sort replay
  // assumes keys that IEEE `<` orders totally.
  k_check_finite<<<(n + 255) / 256, 256, 0, st>>>(d_triangles, n, ctr + 2, kNonFinite);
  if (cudaGetLastError() != cudaSuccess) return drain(RT_ERR_CUDA);
  if (cudaMemcpyAsync(h.flags, ctr, sizeof(h.flags), cudaMemcpyDeviceToHost, st) != cudaSuccess)
    return drain(RT_ERR_CUDA);
  if (cudaStreamSynchronize(st) != cudaSuccess) return RT_ERR_CUDA;
  if (h.flags[2] & kNonFinite) return RT_ERR_INVALID_SCENE;
  k_iota<<<(n + 255) / 256, 256, 0, st>>>(idx, n);
  for (uint32_t L = 0; L < h.levels; L++) {
    uint32_t s0 = h.level_off[L], s1 = h.level_off[L + 1];
    uint32_t ns = s1 - s0;
    if (ns == 0) continue;
    const Seg *ls = dsegs + s0;
    // Queue count and head start at zero for every level; keep the error word.
    if (cudaMemsetAsync(ctr, 0, sizeof(uint32_t) * 2, st) != cudaSuccess) return drain(RT_ERR_CUDA);
    k_keys<<<(n + 255) / 256, 256, 0, st>>>(ls, ns, d_triangles, idx, key, n);
    k_enqueue<<<(ns + 255) / 256, 256, 0, st>>>(ls, ns, queue, ctr);
    uint32_t maxn = 0;
    for (uint32_t j = s0; j < s1; j++) maxn = std::max(maxn, h.segs[j].n);
    if (maxn > kWarpMax) k_sort_big<<<ns, kBigThreads, 0, st>>>(ls, key, idx, P, Q, queue, ctr, ctr + 2);
    k_sort_warps<<<(uint32_t)sms * 8u, 256, 0, st>>>(key, idx, P, Q, queue, ctr, ctr + 1, ctr + 2);
  }
  k_leaves<<<(h.nleaves + 255) / 256, 256, 0, st>>>(dleaves, h.nleaves, idx, d_triangles, d_nodes);
  for (int L = (int)h.levels - 1; L >= 0; L--) {
    uint32_t s0 = h.level_off[L], s1 = h.level_off[L + 1];
    if (s1 > s0) k_inner<<<(s1 - s0 + 255) / 256, 256, 0, st>>>(dsegs + s0, s1 - s0, d_nodes);
  }
  if (cudaGetLastError() != cudaSuccess) return drain(RT_ERR_CUDA);
  if (cudaMemcpyAsync(h.flags, ctr, sizeof(h.flags), cudaMemcpyDeviceToHost, st) != cudaSuccess)
    return drain(RT_ERR_CUDA);
  if (cudaStreamSynchronize(st) != cudaSuccess) return RT_ERR_CUDA;
  return h.flags[2] ? RT_ERR_INTERNAL : RT_SUCCESS;
}
