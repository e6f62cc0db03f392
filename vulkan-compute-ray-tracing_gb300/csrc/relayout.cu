// Traversal layout derived from the reference node array (Bvh.h layout).
//
// The reference traverses its 48-byte nodes one at a time and reads a node's
// box when the node itself is popped (ray-trace-compute.comp:280-307), so a
// visit costs a dependent load per child. Here each inner node stores the
// boxes of BOTH children (64 bytes, four 16-byte loads), so one fetch decides
// which children to descend into, and leaves point straight at a
// precomputed triangle record. The tree itself — every box, every split —
// is the reference's, unchanged.
//
// Inner nodes keep the reference's relative order (rank among inner nodes);
// leaves are numbered by rank among leaves, and tpre/leaf_tri are stored in
// that order so neighbouring leaves sit in neighbouring records.
#include <cuda_runtime.h>

#include "rt_internal.h"
#include "rt_math.cuh"

namespace rtgb {
namespace {

constexpr int kScanBlock = 1024;

__global__ void k_flags(const rt_bvh_node *nodes, uint32_t n, uint32_t *flag) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) flag[i] = nodes[i].left != -1 ? 1u : 0u;
}

// Block-local exclusive scan; writes the block total to sums[blockIdx.x].
__global__ void k_scan_local(const uint32_t *in, uint32_t *out, uint32_t *sums, uint32_t n) {
  __shared__ uint32_t warp_tot[32];
  uint32_t i = blockIdx.x * kScanBlock + threadIdx.x;
  uint32_t v = i < n ? in[i] : 0u;
  uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
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
  uint32_t incl = x + (warp > 0 ? warp_tot[warp - 1] : 0u);
  if (i < n) out[i] = incl - v;
  if (threadIdx.x == kScanBlock - 1) sums[blockIdx.x] = incl;
}

// Exclusive scan of the block totals in place (one block, serial over chunks).
__global__ void k_scan_sums(uint32_t *sums, uint32_t nb) {
  __shared__ uint32_t warp_tot[32];
  __shared__ uint32_t carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (uint32_t base = 0; base < nb; base += kScanBlock) {
    uint32_t i = base + threadIdx.x;
    uint32_t v = i < nb ? sums[i] : 0u;
    uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
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
    uint32_t incl = x + (warp > 0 ? warp_tot[warp - 1] : 0u);
    uint32_t c = carry;
    if (i < nb) sums[i] = c + incl - v;
    __syncthreads();
    if (threadIdx.x == kScanBlock - 1) carry = c + incl;
    __syncthreads();
  }
}

__global__ void k_scan_add(uint32_t *out, const uint32_t *sums, uint32_t n) {
  uint32_t i = blockIdx.x * kScanBlock + threadIdx.x;
  if (i < n) out[i] += sums[blockIdx.x];
}

// Visiting order of a node's two children for each sign octant of a ray
// (bit o set: child 1 first for rays whose direction has sign bits o, bit 0
// x < 0, bit 1 y < 0, bit 2 z < 0): the child whose box centre lies nearer
// along the octant's diagonal goes first. Measured on the 1.31M-triangle
// displaced icosphere against ordering by each ray's own entry distances:
// 1.5% fewer node steps and 3% fewer triangle tests for camera packets, 3.4%
// and 5.7% fewer for single incoherent rays (overlapping boxes make entry
// distances a poor guide), and the traversal loops need no distance at all.
__device__ __forceinline__ uint32_t pair_order(const rt_bvh_node &c0, const rt_bvh_node &c1) {
  const float dx = (c0.min[0] + c0.max[0]) - (c1.min[0] + c1.max[0]);
  const float dy = (c0.min[1] + c0.max[1]) - (c1.min[1] + c1.max[1]);
  const float dz = (c0.min[2] + c0.max[2]) - (c1.min[2] + c1.max[2]);
  uint32_t bits = 0;
  for (int o = 0; o < 8; o++) {
    const float s = ((o & 1) ? -dx : dx) + ((o & 2) ? -dy : dy) + ((o & 4) ? -dz : dz);
    if (s > 0.0f) bits |= 1u << o;
  }
  return bits;
}

__global__ void k_emit(const rt_bvh_node *nodes, uint32_t n, const rt_triangle *tris, const uint32_t *inner_rank,
                       float4 *bvh2, float4 *tpre, int32_t *leaf_tri) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const rt_bvh_node nd = nodes[i];
  if (nd.left != -1) {
    const rt_bvh_node c0 = nodes[nd.left], c1 = nodes[nd.right];
    auto ref = [&](int32_t c, const rt_bvh_node &cn) -> int32_t {
      uint32_t r = inner_rank[c];
      return cn.left != -1 ? (int32_t)r : ~(int32_t)((uint32_t)c - r);
    };
    float4 *o = bvh2 + 4ull * inner_rank[i];
    const float order = __uint_as_float(pair_order(c0, c1));
    o[0] = make_float4(c0.min[0], c0.min[1], c0.max[0], c0.max[1]);
    o[1] = make_float4(c0.min[2], c0.max[2], __int_as_float(ref(nd.left, c0)), order);
    o[2] = make_float4(c1.min[0], c1.min[1], c1.max[0], c1.max[1]);
    o[3] = make_float4(c1.min[2], c1.max[2], __int_as_float(ref(nd.right, c1)), order);
  } else {
    uint32_t k = i - inner_rank[i];
    const rt_triangle t = tris[nd.object];
    f3 v0 = ld3(t.v0), v1 = ld3(t.v1), v2 = ld3(t.v2);
    f3 a = sub3(v0, v1), b = sub3(v2, v0);
    f3 nn = cross3(b, a);
    float4 *o = tpre + 3ull * k;
    o[0] = make_float4(v0.x, v0.y, v0.z, nn.x);
    o[1] = make_float4(nn.y, nn.z, a.x, a.y);
    o[2] = make_float4(a.z, b.x, b.y, b.z);
    leaf_tri[k] = nd.object;
  }
}

}  // namespace

// Exclusive scan of n uint32 values (in may equal out). `sums` needs
// ceil(n / 1024) words.
cudaError_t exclusive_scan_u32(const uint32_t *in, uint32_t *out, uint32_t *sums, uint32_t n, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  uint32_t nb = (n + kScanBlock - 1) / kScanBlock;
  k_scan_local<<<nb, kScanBlock, 0, st>>>(in, out, sums, n);
  k_scan_sums<<<1, kScanBlock, 0, st>>>(sums, nb);
  k_scan_add<<<nb, kScanBlock, 0, st>>>(out, sums, n);
  return cudaGetLastError();
}

cudaError_t launch_relayout(const rt_bvh_node *nodes, uint32_t nnodes, const rt_triangle *tris, float4 *bvh2,
                            float4 *tpre, int32_t *leaf_tri, uint32_t *scratch, cudaStream_t st) {
  uint32_t *rank = scratch;
  uint32_t *sums = scratch + nnodes;
  const int B = 256;
  k_flags<<<(nnodes + B - 1) / B, B, 0, st>>>(nodes, nnodes, rank);
  cudaError_t e = exclusive_scan_u32(rank, rank, sums, nnodes, st);
  if (e != cudaSuccess) return e;
  k_emit<<<(nnodes + B - 1) / B, B, 0, st>>>(nodes, nnodes, tris, rank, bvh2, tpre, leaf_tri);
  return cudaGetLastError();
}

}  // namespace rtgb
