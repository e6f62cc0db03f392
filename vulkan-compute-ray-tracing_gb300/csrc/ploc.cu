// Alternative tree: bottom-up agglomerative clustering (PLOC: Meister and
// Bittner, "Parallel Locally-Ordered Clustering for Bounding Volume
// Hierarchy Construction", IEEE TVCG 2018), built on the GPU and emitted in
// the Bvh.h node layout, one triangle per leaf.
//
// Triangles start as clusters in Morton order (lbvh.cu's key). Each round,
// every cluster finds, among the `radius` clusters on either side, the one
// whose merged box has the smallest surface area; mutually nearest pairs
// merge into a new inner node; the survivors are compacted in order. Rounds
// repeat until one cluster (the root) is left. The trees approach
// surface-area-heuristic quality, far tighter than the reference's
// random-axis median splits — a separately reported mode ("bvh.builder" =
// 2), not a replacement for the reference's tree.
#include <cuda_runtime.h>

#include <cstdio>

#include "rt_internal.h"

namespace rtgb {

namespace {

struct Box {
  float lo[3], hi[3];
};

__device__ __forceinline__ float half_area(const Box &b) {
  float dx = b.hi[0] - b.lo[0], dy = b.hi[1] - b.lo[1], dz = b.hi[2] - b.lo[2];
  return dx * dy + dy * dz + dz * dx;
}

__device__ __forceinline__ Box join(const Box &a, const Box &b) {
  Box r;
  for (int k = 0; k < 3; k++) {
    r.lo[k] = fminf(a.lo[k], b.lo[k]);
    r.hi[k] = fmaxf(a.hi[k], b.hi[k]);
  }
  return r;
}

// Leaves: cluster k = triangle idx[k] in Morton order, node n-1+k.
__global__ void k_ploc_leaves(const rt_triangle *__restrict__ tris, const uint32_t *__restrict__ idx, uint32_t n,
                              Box *boxes, int32_t *ids, uint32_t *heights, rt_bvh_node *nodes) {
  uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const uint32_t o = idx[k];
  const rt_triangle t = tris[o];
  Box b;
  rt_bvh_node nd;
  for (int a = 0; a < 3; a++) {
    float lo = (t.v1[a] < t.v0[a]) ? t.v1[a] : t.v0[a];
    lo = (t.v2[a] < lo) ? t.v2[a] : lo;
    float hi = (t.v0[a] < t.v1[a]) ? t.v1[a] : t.v0[a];
    hi = (hi < t.v2[a]) ? t.v2[a] : hi;
    b.lo[a] = nd.min[a] = __fsub_rn(lo, 0.0001f);
    b.hi[a] = nd.max[a] = __fadd_rn(hi, 0.0001f);
  }
  nd._pad0 = 0.0f;
  nd.left = -1;
  nd.right = -1;
  nd.object = (int32_t)o;
  nd._pad1[0] = nd._pad1[1] = 0;
  const uint32_t node = n - 1 + k;
  nodes[node] = nd;
  boxes[k] = b;
  ids[k] = (int32_t)node;
  heights[k] = 1;
}

// Tie key of the unordered pair (i, j), the same seen from either side:
// nearer positions first, then pairs starting at an even position (so that a
// run of equal boxes pairs up as (0, 1), (2, 3), ... and halves each round
// instead of merging one pair per round into a chain), then the lower start.
__device__ __forceinline__ unsigned long long pair_key(uint32_t i, uint32_t j) {
  const uint32_t lo = min(i, j), gap = max(i, j) - lo;
  return ((unsigned long long)gap << 33) | ((unsigned long long)(lo & 1u) << 32) | lo;
}

// Nearest neighbour by merged surface area within the radius, equal areas
// ordered by pair_key. Area and key are symmetric in the pair, so the pair
// smallest in (area, key) among all is chosen by both its members: every
// round merges at least one pair.
__global__ void k_ploc_nearest(const Box *__restrict__ boxes, uint32_t m, uint32_t radius, uint32_t *nn) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  const Box bi = boxes[i];
  float best = __int_as_float(0x7f800000);
  unsigned long long best_key = ~0ull;
  uint32_t arg = i;
  const uint32_t lo = i > radius ? i - radius : 0;
  const uint32_t hi = min(m - 1, i + radius);
  for (uint32_t j = lo; j <= hi; j++) {
    if (j == i) continue;
    const float a = half_area(join(bi, boxes[j]));
    const unsigned long long key = pair_key(i, j);
    if (arg == i || a < best || (a == best && key < best_key)) {
      best = a;
      best_key = key;
      arg = j;
    }
  }
  nn[i] = arg;
}

// keep[i] = 1 if cluster i survives this round (merged into it or untouched);
// merge[i] = 1 if it is the lower partner of a mutual pair.
__global__ void k_ploc_flags(const uint32_t *__restrict__ nn, uint32_t m, uint32_t *keep, uint32_t *merge) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  uint32_t j = nn[i];
  bool mutual = j != i && nn[j] == i;
  merge[i] = (mutual && i < j) ? 1u : 0u;
  keep[i] = (!mutual || i < j) ? 1u : 0u;
}

__global__ void k_ploc_merge(const Box *__restrict__ boxes, const int32_t *__restrict__ ids,
                             const uint32_t *__restrict__ heights, const uint32_t *__restrict__ nn,
                             const uint32_t *__restrict__ keep_pos, const uint32_t *__restrict__ keep,
                             const uint32_t *__restrict__ merge_pos, const uint32_t *__restrict__ merge, uint32_t m,
                             int32_t next_id_top, Box *boxes_out, int32_t *ids_out, uint32_t *heights_out,
                             rt_bvh_node *nodes) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m || !keep[i]) return;
  Box b = boxes[i];
  int32_t id = ids[i];
  uint32_t h = heights[i];
  if (merge[i]) {
    const uint32_t j = nn[i];
    const Box bj = boxes[j];
    b = join(b, bj);
    // Inner nodes are numbered down from n-2 so the final merge is node 0.
    const int32_t nid = next_id_top - (int32_t)merge_pos[i];
    rt_bvh_node nd;
    for (int k = 0; k < 3; k++) {
      nd.min[k] = b.lo[k];
      nd.max[k] = b.hi[k];
    }
    nd._pad0 = 0.0f;
    nd.left = id;
    nd.right = ids[j];
    nd.object = -1;
    nd._pad1[0] = nd._pad1[1] = 0;
    nodes[nid] = nd;
    id = nid;
    h = 1 + max(h, heights[j]);
  }
  const uint32_t o = keep_pos[i];
  boxes_out[o] = b;
  ids_out[o] = id;
  heights_out[o] = h;
}

}  // namespace

rt_status gpu_build_ploc(const rt_triangle *d_tris, uint32_t n, uint32_t radius, rt_bvh_node *d_nodes,
                         cudaStream_t st, float *ms_out, uint32_t *depth_out, char *errbuf, size_t errlen) {
  if (n == 0 || radius < 1 || radius > 256) return RT_ERR_INVALID_ARGUMENT;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  // Scratch, in 32-bit words: the Morton sort | boxes 2 x 6n | ids 2n |
  // heights 2n | nn, keep, merge, keep_pos, merge_pos 5n | scan sums.
  const size_t sort_words = lbvh_sorted_keys_words(n);
  const size_t words = sort_words + 2 * 6ull * n + 2ull * n + 2ull * n + 5ull * n + (n / 1024 + 8);
  void *mem = nullptr;
  cudaError_t e = cudaMallocAsync(&mem, 4 * words, st);
  if (e != cudaSuccess) {
    std::snprintf(errbuf, errlen, "ploc scratch: %s", cudaGetErrorString(e));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return RT_ERR_OUT_OF_MEMORY;
  }
  uint32_t *w = static_cast<uint32_t *>(mem);
  uint32_t *sortbuf = w;
  Box *boxes[2] = {reinterpret_cast<Box *>(w + sort_words), reinterpret_cast<Box *>(w + sort_words + 6ull * n)};
  uint32_t *p = w + sort_words + 12ull * n;
  int32_t *ids[2] = {reinterpret_cast<int32_t *>(p), reinterpret_cast<int32_t *>(p + n)};
  p += 2ull * n;
  uint32_t *heights[2] = {p, p + n};
  p += 2ull * n;
  uint32_t *nn = p, *keep = p + n, *merge = p + 2ull * n, *keep_pos = p + 3ull * n, *merge_pos = p + 4ull * n;
  p += 5ull * n;
  uint32_t *sums = p;
  rt_status status = RT_SUCCESS;
  uint32_t *codes = nullptr, *idx = nullptr;
  cudaEventRecord(e0, st);
  const uint32_t B = 256;
  uint32_t m = n, cur = 0;
  int32_t top = (int32_t)n - 2;  // next inner node id (counting down)
  uint32_t rounds = 0;
  uint32_t depth = 1;
  e = lbvh_sorted_keys(d_tris, n, sortbuf, &codes, &idx, st);
  if (e == cudaSuccess) {
    k_ploc_leaves<<<(n + B - 1) / B, B, 0, st>>>(d_tris, idx, n, boxes[0], ids[0], heights[0], d_nodes);
    e = cudaGetLastError();
  }
  while (e == cudaSuccess && m > 1) {
    if (++rounds > n) {  // each round removes at least one cluster
      status = RT_ERR_INTERNAL;
      std::snprintf(errbuf, errlen, "ploc: no progress");
      break;
    }
    const uint32_t G = (m + B - 1) / B;
    k_ploc_nearest<<<G, B, 0, st>>>(boxes[cur], m, radius, nn);
    k_ploc_flags<<<G, B, 0, st>>>(nn, m, keep, merge);
    if ((e = exclusive_scan_u32(keep, keep_pos, sums, m, st)) != cudaSuccess) break;
    if ((e = exclusive_scan_u32(merge, merge_pos, sums, m, st)) != cudaSuccess) break;
    k_ploc_merge<<<G, B, 0, st>>>(boxes[cur], ids[cur], heights[cur], nn, keep_pos, keep, merge_pos, merge, m, top,
                                  boxes[cur ^ 1], ids[cur ^ 1], heights[cur ^ 1], d_nodes);
    // Survivors and merges of this round, read back to size the next one.
    uint32_t h[4];
    cudaMemcpyAsync(&h[0], keep_pos + m - 1, 4, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(&h[1], keep + m - 1, 4, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(&h[2], merge_pos + m - 1, 4, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(&h[3], merge + m - 1, 4, cudaMemcpyDeviceToHost, st);
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) break;
    const uint32_t survivors = h[0] + h[1], merges = h[2] + h[3];
    if (merges == 0 || survivors + merges != m) {
      status = RT_ERR_INTERNAL;
      std::snprintf(errbuf, errlen, "ploc: inconsistent round (%u survivors, %u merges of %u)", survivors, merges, m);
      break;
    }
    top -= (int32_t)merges;
    m = survivors;
    cur ^= 1;
  }
  if (e == cudaSuccess && status == RT_SUCCESS) {
    cudaMemcpyAsync(&depth, heights[cur], 4, cudaMemcpyDeviceToHost, st);
    e = cudaStreamSynchronize(st);
  }
  cudaEventRecord(e1, st);
  cudaStreamSynchronize(st);
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaFreeAsync(mem, st);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (e != cudaSuccess) {
    std::snprintf(errbuf, errlen, "ploc build: %s", cudaGetErrorString(e));
    return RT_ERR_CUDA;
  }
  if (status != RT_SUCCESS) return status;
  if (top != -1) {
    std::snprintf(errbuf, errlen, "ploc build: %d inner nodes unassigned", top + 1);
    return RT_ERR_INTERNAL;
  }
  if (ms_out) *ms_out = ms;
  if (depth_out) *depth_out = depth;
  return RT_SUCCESS;
}

}  // namespace rtgb
