// Ray reordering for closest-hit casting ("trace.sort") and, on request,
// for the bounces of wavefront renders ("render.sort").
//
// Rays whose origins and directions are close visit the same BVH nodes; a
// warp holding such rays diverges less and shares cache lines. The batch is
// bucketed by a 20-bit Morton code over five coordinates — origin x, y, z
// normalised to the batch's extent and the direction's octahedral (u, v)
// — where only coordinates that vary across the batch receive bits (a
// camera batch shares one origin, so all 20 bits go to the direction). A
// counting sort over the 2^20 buckets produces a permutation; the caster
// then reads rays through it and writes each hit back to its input slot.
// Order inside a bucket is arbitrary; results do not depend on the order.
// With a device-side count (d_n), only the first *d_n rays of the buffer
// take part (the launch is sized for the buffer's capacity n). On request
// the sorted batch is also cut into cell tiles (RayCells) for the beam
// caster.
#include <cuda_runtime.h>

#include "rt_internal.h"

namespace rtgb {
namespace {

constexpr int kBits = 20;
constexpr uint32_t kBuckets = 1u << kBits;

// float <-> order-preserving uint for atomic min/max
__device__ __forceinline__ uint32_t f2o(float f) {
  uint32_t u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float o2f(uint32_t u) {
  return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

__device__ __forceinline__ void octa(float dx, float dy, float dz, float &u, float &v) {
  float s = fabsf(dx) + fabsf(dy) + fabsf(dz);
  s = s > 0.0f ? 1.0f / s : 0.0f;
  float px = dx * s, py = dy * s;
  if (dz < 0.0f) {
    float qx = (1.0f - fabsf(py)) * (px >= 0.0f ? 1.0f : -1.0f);
    float qy = (1.0f - fabsf(px)) * (py >= 0.0f ? 1.0f : -1.0f);
    px = qx;
    py = qy;
  }
  u = px;
  v = py;
}

__device__ __forceinline__ void ray_coords(const float4 *rays, uint32_t i, float c[5]) {
  float4 a = __ldg(rays + 2ull * i), b = __ldg(rays + 2ull * i + 1);
  c[0] = a.x;
  c[1] = a.y;
  c[2] = a.z;
  octa(b.x, b.y, b.z, c[3], c[4]);
}

// ext[0..4] = ordered min, ext[5..9] = ordered max (initialised by the host),
// over one ray in kExtentStride: the extent only scales the Morton key, and
// rays outside the sampled extent clamp to the edge buckets (the order only
// affects speed, never results), so the pass reads an eighth of the rays.
constexpr uint32_t kExtentStride = 8;
__global__ void k_extent(const float4 *__restrict__ rays, uint32_t n, const uint32_t *d_n, uint32_t *ext) {
  if (d_n) n = min(n, *d_n);
  float lo[5], hi[5];
  for (int k = 0; k < 5; k++) {
    lo[k] = __int_as_float(0x7f800000);
    hi[k] = -__int_as_float(0x7f800000);
  }
  for (uint64_t i = (uint64_t)(blockIdx.x * blockDim.x + threadIdx.x) * kExtentStride; i < n;
       i += (uint64_t)gridDim.x * blockDim.x * kExtentStride) {
    float c[5];
    ray_coords(rays, i, c);
    for (int k = 0; k < 5; k++) {
      lo[k] = fminf(lo[k], c[k]);
      hi[k] = fmaxf(hi[k], c[k]);
    }
  }
  for (int k = 0; k < 5; k++) {
    for (int o = 16; o > 0; o >>= 1) {
      lo[k] = fminf(lo[k], __shfl_xor_sync(0xffffffffu, lo[k], o));
      hi[k] = fmaxf(hi[k], __shfl_xor_sync(0xffffffffu, hi[k], o));
    }
  }
  if ((threadIdx.x & 31) == 0) {
    for (int k = 0; k < 5; k++) {
      if (hi[k] >= lo[k]) {
        atomicMin(ext + k, f2o(lo[k]));
        atomicMax(ext + 5 + k, f2o(hi[k]));
      }
    }
  }
}

__device__ __forceinline__ uint32_t ray_key(const float4 *rays, uint32_t i, const uint32_t *ext) {
  float c[5];
  ray_coords(rays, i, c);
  // Bits per coordinate: only coordinates with a nonzero extent take part.
  int active[5], na = 0;
  float lo[5], scale[5];
  for (int k = 0; k < 5; k++) {
    lo[k] = o2f(ext[k]);
    float span = o2f(ext[5 + k]) - lo[k];
    scale[k] = span > 1e-12f ? 1.0f / span : 0.0f;
    if (span > 1e-12f) active[na++] = k;
  }
  if (na == 0) return 0;
  int bits = kBits / na;
  uint32_t q[5];
  for (int j = 0; j < na; j++) {
    int k = active[j];
    float t = (c[k] - lo[k]) * scale[k];
    t = fminf(fmaxf(t, 0.0f), 0.99999994f);
    q[j] = (uint32_t)(t * (float)(1u << bits));
  }
  uint32_t key = 0;
  for (int b = bits - 1; b >= 0; b--)
    for (int j = 0; j < na; j++) key = (key << 1) | ((q[j] >> b) & 1u);
  return key;
}

__global__ void k_hist(const float4 *__restrict__ rays, uint32_t n, const uint32_t *d_n, const uint32_t *ext,
                       uint32_t *keys, uint32_t *hist) {
  if (d_n) n = min(n, *d_n);
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint32_t k = ray_key(rays, i, ext);
  keys[i] = k;
  atomicAdd(hist + k, 1u);
}

__global__ void k_scatter(const uint32_t *__restrict__ keys, uint32_t n, const uint32_t *d_n, uint32_t *offsets,
                          uint32_t *perm) {
  if (d_n) n = min(n, *d_n);
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint32_t slot = atomicAdd(offsets + keys[i], 1u);
  perm[slot] = i;
}

__global__ void k_init_ext(uint32_t *ext) {
  int k = threadIdx.x;
  if (k < 5) {
    ext[k] = 0xffffffffu;
    ext[5 + k] = 0u;
  }
}

// Cells: runs of 64 consecutive buckets (a Morton-aligned 8 x 8 block of
// direction buckets in a one-origin batch). After the scatter hist[k] is
// one past bucket k's last sorted position, so cell c spans
// [hist[64c - 1], hist[64c + 63]). Each cell is cut into tiles of at most
// kTileRays rays.
constexpr uint32_t kCellBuckets = 64;
constexpr uint32_t kCells = kBuckets / kCellBuckets;
constexpr uint32_t kTileRays = 256;

__device__ __forceinline__ void cell_span(const uint32_t *hist, uint32_t c, uint32_t &b, uint32_t &e) {
  b = c ? hist[c * kCellBuckets - 1] : 0u;
  e = hist[c * kCellBuckets + kCellBuckets - 1];
}

__global__ void k_cell_count(const uint32_t *__restrict__ hist, uint32_t *cnt) {
  const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= kCells) return;
  uint32_t b, e;
  cell_span(hist, c, b, e);
  cnt[c] = (e - b + kTileRays - 1) / kTileRays;
}

__global__ void k_cell_emit(const uint32_t *__restrict__ hist, const uint32_t *__restrict__ cnt,
                            const uint32_t *__restrict__ off, uint32_t *tiles, uint32_t *count) {
  const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= kCells) return;
  uint32_t b, e;
  cell_span(hist, c, b, e);
  for (uint32_t j = 0; j < cnt[c]; j++) {
    const uint32_t t0 = b + j * kTileRays;
    tiles[2 * (off[c] + j)] = t0;
    tiles[2 * (off[c] + j) + 1] = min(t0 + kTileRays, e);
  }
  if (c == kCells - 1) *count = off[c] + cnt[c];
}

size_t cell_words(uint32_t n) {
  // counts | offsets | scan sums | tile count | tiles (at most one partial per cell)
  return 2ull * kCells + (kCells / 1024 + 2) + 1 + 2ull * (kCells + n / kTileRays + 1);
}

}  // namespace

size_t raysort_scratch_bytes(uint32_t n) {
  // ext (16 words) | keys n | hist kBuckets | scan sums | perm n | cell tiles
  return 4ull * (16 + n + kBuckets + (kBuckets / 1024 + 2) + n + cell_words(n));
}

cudaError_t launch_raysort(const rt_ray *rays, uint32_t n, const uint32_t *d_n, void *scratch, uint32_t **perm_out,
                           cudaStream_t st, RayCells *cells) {
  uint32_t *ext = static_cast<uint32_t *>(scratch);
  uint32_t *keys = ext + 16;
  uint32_t *hist = keys + n;
  uint32_t *sums = hist + kBuckets;
  uint32_t *perm = sums + (kBuckets / 1024 + 2);
  *perm_out = perm;
  const float4 *r = reinterpret_cast<const float4 *>(rays);
  k_init_ext<<<1, 32, 0, st>>>(ext);
  k_extent<<<304, 256, 0, st>>>(r, n, d_n, ext);
  cudaError_t e = cudaMemsetAsync(hist, 0, 4ull * kBuckets, st);
  if (e != cudaSuccess) return e;
  k_hist<<<(n + 255) / 256, 256, 0, st>>>(r, n, d_n, ext, keys, hist);
  e = exclusive_scan_u32(hist, hist, sums, kBuckets, st);
  if (e != cudaSuccess) return e;
  k_scatter<<<(n + 255) / 256, 256, 0, st>>>(keys, n, d_n, hist, perm);
  if (!cells) return cudaGetLastError();
  uint32_t *cnt = perm + n, *off = cnt + kCells, *csums = off + kCells, *count = csums + (kCells / 1024 + 2);
  uint32_t *tiles = count + 1;
  k_cell_count<<<kCells / 256, 256, 0, st>>>(hist, cnt);
  e = exclusive_scan_u32(cnt, off, csums, kCells, st);
  if (e != cudaSuccess) return e;
  k_cell_emit<<<kCells / 256, 256, 0, st>>>(hist, cnt, off, tiles, count);
  cells->ext = ext;
  cells->tiles = tiles;
  cells->count = count;
  return cudaGetLastError();
}

}  // namespace rtgb
