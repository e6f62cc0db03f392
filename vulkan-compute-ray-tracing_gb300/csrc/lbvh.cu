// Alternative tree: a linear BVH over triangle centroids, built on the GPU
// (Karras, "Maximizing Parallelism in the Construction of BVHs, Octrees,
// and k-d Trees", HPG 2012), emitted in the same Bvh.h node layout so the
// re-layout and every traversal kernel run on it unchanged.
//
// The reference's tree splits every node at the median along a random axis
// (Bvh.h:160-175); sibling boxes overlap heavily and a ray visits hundreds of
// nodes. Closest-hit results do not depend on the tree (only the order in
// which equal-t candidates are met does), so a tighter tree is a separate,
// separately reported mode ("bvh.builder" = 1), not a replacement.
//
// Steps: centroid bounds -> 30-bit Morton code per triangle -> stable radix
// sort (one bit per pass, scan-based split) -> one thread per inner node
// finds its key range and split from the longest common prefixes of
// neighbouring (code, index) keys -> leaves walk to the root with an atomic
// visit count per inner node; the second child to arrive writes the union.
// Leaf boxes are padded by 1e-4 exactly as Bvh.h pads them (Bvh.h:94-98).
#include <cuda_runtime.h>

#include <cstdio>

#include "rt_internal.h"

namespace rtgb {
namespace {

__device__ __forceinline__ uint32_t f2o(float f) {
  uint32_t u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float o2f(uint32_t u) {
  return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

__device__ __forceinline__ float3 centroid(const rt_triangle &t) {
  return make_float3((t.v0[0] + t.v1[0] + t.v2[0]) * (1.0f / 3.0f), (t.v0[1] + t.v1[1] + t.v2[1]) * (1.0f / 3.0f),
                     (t.v0[2] + t.v1[2] + t.v2[2]) * (1.0f / 3.0f));
}

__global__ void k_init_bounds(uint32_t *ext) {
  if (threadIdx.x < 3) {
    ext[threadIdx.x] = 0xffffffffu;
    ext[3 + threadIdx.x] = 0u;
  }
}

__global__ void k_bounds(const rt_triangle *__restrict__ tris, uint32_t n, uint32_t *ext) {
  float lo[3] = {3.4e38f, 3.4e38f, 3.4e38f}, hi[3] = {-3.4e38f, -3.4e38f, -3.4e38f};
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    float3 c = centroid(tris[i]);
    lo[0] = fminf(lo[0], c.x);
    lo[1] = fminf(lo[1], c.y);
    lo[2] = fminf(lo[2], c.z);
    hi[0] = fmaxf(hi[0], c.x);
    hi[1] = fmaxf(hi[1], c.y);
    hi[2] = fmaxf(hi[2], c.z);
  }
  for (int k = 0; k < 3; k++) {
    for (int o = 16; o > 0; o >>= 1) {
      lo[k] = fminf(lo[k], __shfl_xor_sync(0xffffffffu, lo[k], o));
      hi[k] = fmaxf(hi[k], __shfl_xor_sync(0xffffffffu, hi[k], o));
    }
  }
  if ((threadIdx.x & 31) == 0)
    for (int k = 0; k < 3; k++) {
      atomicMin(ext + k, f2o(lo[k]));
      atomicMax(ext + 3 + k, f2o(hi[k]));
    }
}

__device__ __forceinline__ uint32_t spread10(uint32_t v) {
  v &= 1023u;
  v = (v | (v << 16)) & 0x030000FFu;
  v = (v | (v << 8)) & 0x0300F00Fu;
  v = (v | (v << 4)) & 0x030C30C3u;
  v = (v | (v << 2)) & 0x09249249u;
  return v;
}

__global__ void k_morton(const rt_triangle *__restrict__ tris, uint32_t n, const uint32_t *ext, uint32_t *codes,
                         uint32_t *idx) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float3 c = centroid(tris[i]);
  float p[3] = {c.x, c.y, c.z};
  uint32_t q[3];
  for (int k = 0; k < 3; k++) {
    float lo = o2f(ext[k]), span = o2f(ext[3 + k]) - lo;
    float t = span > 0.0f ? (p[k] - lo) / span : 0.0f;
    t = fminf(fmaxf(t, 0.0f), 1.0f);
    q[k] = min(1023u, (uint32_t)(t * 1024.0f));
  }
  codes[i] = (spread10(q[0]) << 2) | (spread10(q[1]) << 1) | spread10(q[2]);
  idx[i] = i;
}

__global__ void k_bitflag(const uint32_t *__restrict__ codes, uint32_t n, int bit, uint32_t *flag) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) flag[i] = ((codes[i] >> bit) & 1u) ? 0u : 1u;
}

// Stable split: keys with the bit clear keep their order first, then the rest.
__global__ void k_split(const uint32_t *__restrict__ codes, const uint32_t *__restrict__ idx,
                        const uint32_t *__restrict__ flag, const uint32_t *__restrict__ pos, uint32_t n,
                        uint32_t *codes_out, uint32_t *idx_out) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t zeros = pos[n - 1] + flag[n - 1];
  uint32_t dst = flag[i] ? pos[i] : zeros + (i - pos[i]);
  codes_out[dst] = codes[i];
  idx_out[dst] = idx[i];
}

// Longest common prefix of the keys (code, position) at i and j; -1 outside.
__device__ __forceinline__ int delta(const uint32_t *codes, int n, int i, int j) {
  if (j < 0 || j >= n) return -1;
  uint32_t a = codes[i], b = codes[j];
  if (a != b) return __clz(a ^ b);
  return 32 + __clz((uint32_t)i ^ (uint32_t)j);
}

__global__ void k_karras(const uint32_t *__restrict__ codes, int n, int32_t *left, int32_t *right, int32_t *parent) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n - 1) return;
  int d = (delta(codes, n, i, i + 1) - delta(codes, n, i, i - 1)) >= 0 ? 1 : -1;
  int dmin = delta(codes, n, i, i - d);
  int lmax = 2;
  while (delta(codes, n, i, i + lmax * d) > dmin) lmax <<= 1;
  int l = 0;
  for (int t = lmax >> 1; t >= 1; t >>= 1)
    if (delta(codes, n, i, i + (l + t) * d) > dmin) l += t;
  int j = i + l * d;
  int dnode = delta(codes, n, i, j);
  int s = 0;
  for (int t = (l + 1) >> 1;; t = (t + 1) >> 1) {
    if (delta(codes, n, i, i + (s + t) * d) > dnode) s += t;
    if (t == 1) break;
  }
  int g = i + s * d + (d < 0 ? -1 : 0);
  int lo = i < j ? i : j, hi = i < j ? j : i;
  // Inner nodes are 0..n-2, leaf k is node n-1+k.
  int L = (lo == g) ? (n - 1 + g) : g;
  int R = (hi == g + 1) ? (n - 1 + g + 1) : (g + 1);
  left[i] = L;
  right[i] = R;
  parent[L] = i;
  parent[R] = i;
}

// Node read that bypasses L1: the sibling wrote it from another SM.
__device__ __forceinline__ void load_box_cg(const rt_bvh_node *nd, float lo[3], float hi[3]) {
  const float4 *p = reinterpret_cast<const float4 *>(nd);
  float4 a = __ldcg(p), b = __ldcg(p + 1);
  lo[0] = a.x;
  lo[1] = a.y;
  lo[2] = a.z;
  hi[0] = b.x;
  hi[1] = b.y;
  hi[2] = b.z;
}

constexpr int kMaxWalk = 128;  // longer than any path of a 30-bit-code LBVH (<= 64 levels)

__global__ void k_lbvh_boxes(const rt_triangle *__restrict__ tris, const uint32_t *__restrict__ idx, int n,
                             const int32_t *__restrict__ left, const int32_t *__restrict__ right,
                             const int32_t *__restrict__ parent, uint32_t *visits, rt_bvh_node *nodes,
                             uint32_t *depth_max) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const int leaf = n - 1 + k;
  const uint32_t o = idx[k];
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
  nodes[leaf] = nd;
  int cur = leaf;
  for (int step = 0; cur != 0; step++) {
    int p = parent[cur];
    if (step >= kMaxWalk || p < 0 || p >= n - 1) {
      atomicMax(depth_max, 0xffffffffu);  // malformed: reported as an error by the host
      return;
    }
    __threadfence();
    if (atomicAdd(visits + p, 1u) == 0) break;  // the sibling finishes the parent
    __threadfence();
    float alo[3], ahi[3], blo[3], bhi[3];
    load_box_cg(nodes + left[p], alo, ahi);
    load_box_cg(nodes + right[p], blo, bhi);
    rt_bvh_node q;
    for (int c = 0; c < 3; c++) {
      q.min[c] = fminf(alo[c], blo[c]);
      q.max[c] = fmaxf(ahi[c], bhi[c]);
    }
    q._pad0 = 0.0f;
    q.left = left[p];
    q.right = right[p];
    q.object = -1;
    q._pad1[0] = q._pad1[1] = 0;
    nodes[p] = q;
    cur = p;
  }
  // Levels on this leaf's path (root = 1).
  uint32_t levels = 1;
  for (int c = leaf, step = 0; c != 0 && step < kMaxWalk; c = parent[c], step++) levels++;
  atomicMax(depth_max, levels);
}

}  // namespace

size_t lbvh_sorted_keys_words(uint32_t n) { return 16 + 6ull * n + (n / 1024 + 8); }

// Centroid bounds -> Morton codes -> stable radix sort. `scratch` holds
// lbvh_sorted_keys_words(n) words: bounds 16 | codes 2n | indices 2n |
// flags n | scan n | scan block sums n/1024+8. The sorted codes and triangle
// indices are returned as pointers into it.
cudaError_t lbvh_sorted_keys(const rt_triangle *d_tris, uint32_t n, uint32_t *scratch, uint32_t **codes_out,
                             uint32_t **idx_out, cudaStream_t st) {
  uint32_t *ext = scratch;
  uint32_t *codes[2] = {ext + 16, ext + 16 + n};
  uint32_t *idx[2] = {ext + 16 + 2ull * n, ext + 16 + 3ull * n};
  uint32_t *flag = ext + 16 + 4ull * n;
  uint32_t *pos = flag + n;
  uint32_t *sums = pos + n;
  const uint32_t B = 256, G = (n + B - 1) / B;
  k_init_bounds<<<1, 32, 0, st>>>(ext);
  k_bounds<<<304, 256, 0, st>>>(d_tris, n, ext);
  k_morton<<<G, B, 0, st>>>(d_tris, n, ext, codes[0], idx[0]);
  int cur = 0;
  cudaError_t e = cudaSuccess;
  for (int bit = 0; bit < 30; bit++) {
    k_bitflag<<<G, B, 0, st>>>(codes[cur], n, bit, flag);
    e = exclusive_scan_u32(flag, pos, sums, n, st);
    if (e != cudaSuccess) return e;
    k_split<<<G, B, 0, st>>>(codes[cur], idx[cur], flag, pos, n, codes[cur ^ 1], idx[cur ^ 1]);
    cur ^= 1;
  }
  *codes_out = codes[cur];
  *idx_out = idx[cur];
  return cudaGetLastError();
}

rt_status gpu_build_lbvh(const rt_triangle *d_tris, uint32_t n, rt_bvh_node *d_nodes, cudaStream_t st, float *ms_out,
                         uint32_t *depth_out, char *errbuf, size_t errlen) {
  if (n == 0) return RT_ERR_INVALID_ARGUMENT;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  // Scratch, in 32-bit words: the sort's words | left n | right n |
  // parent 2n | visit counts n | depth 8.
  void *mem = nullptr;
  const size_t sort_words = lbvh_sorted_keys_words(n);
  const size_t words = sort_words + n + n + 2ull * n + n + 8;
  cudaError_t e = cudaMallocAsync(&mem, 4 * words, st);
  if (e != cudaSuccess) {
    std::snprintf(errbuf, errlen, "lbvh scratch: %s", cudaGetErrorString(e));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return RT_ERR_OUT_OF_MEMORY;
  }
  uint32_t *sortbuf = static_cast<uint32_t *>(mem);
  int32_t *left = reinterpret_cast<int32_t *>(sortbuf + sort_words);
  int32_t *right = left + n;
  int32_t *parent = right + n;
  uint32_t *visits = reinterpret_cast<uint32_t *>(parent + 2ull * n);
  uint32_t *dmax = visits + n;
  cudaEventRecord(e0, st);
  const uint32_t B = 256, G = (n + B - 1) / B;
  uint32_t *codes = nullptr, *idx = nullptr;
  e = lbvh_sorted_keys(d_tris, n, sortbuf, &codes, &idx, st);
  if (e == cudaSuccess) {
    cudaMemsetAsync(visits, 0, 4ull * n + 32, st);  // visit counts and the depth word
    cudaMemsetAsync(parent, 0xff, 4ull * 2 * n, st);
    if (n > 1) k_karras<<<(n - 1 + B - 1) / B, B, 0, st>>>(codes, (int)n, left, right, parent);
    k_lbvh_boxes<<<G, B, 0, st>>>(d_tris, idx, (int)n, left, right, parent, visits, d_nodes, dmax);
  }
  cudaEventRecord(e1, st);
  uint32_t depth = 0;
  cudaMemcpyAsync(&depth, dmax, 4, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  float ms = 0.0f;
  if (e == cudaSuccess) cudaEventElapsedTime(&ms, e0, e1);
  cudaFreeAsync(mem, st);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (e != cudaSuccess) {
    std::snprintf(errbuf, errlen, "lbvh build: %s", cudaGetErrorString(e));
    return RT_ERR_CUDA;
  }
  if (depth == 0xffffffffu || depth == 0) {
    std::snprintf(errbuf, errlen, "lbvh build: malformed tree");
    return RT_ERR_INTERNAL;
  }
  if (ms_out) *ms_out = ms;
  if (depth_out) *depth_out = depth;
  return RT_SUCCESS;
}

}  // namespace rtgb
