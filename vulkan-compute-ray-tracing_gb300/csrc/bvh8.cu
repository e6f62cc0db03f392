// 8-wide traversal tree (bvh8) collapsed from the children-pair layout.
//
// The tree is the reference's (or the selected builder's) binary tree with
// levels folded together; no box is recomputed or moved. Each bvh8 node
// holds up to eight children. By default the binary nodes that become bvh8
// nodes are chosen by the surface area heuristic (the SAH collapse below,
// the dynamic program of Ylitie et al., "Efficient Incoherent Ray Traversal
// on GPUs Through Compressed Wide BVHs", HPG 2017, for single-triangle
// leaves). The alternative ("bvh8.collapse" 0) starts from one inner node's
// two children and replaces the inner child with the largest surface area
// by its own two children until there are eight or only leaves are left
// (greedy collapse as in Wald et al., "Getting Rid of Packets", RT 2008); a
// node with fewer than eight children then holds leaves only, which bounds
// the node count by (4n - 1) / 7 for n leaves, the capacity reserved.
//
// Slots are assigned by position (Ylitie et al.'s octant order): slot s,
// read as three bits (x, y, z), stands for the corner of the node on the
// positive side of the axes whose bit is set. Each child goes to the free
// slot whose corner direction best matches the offset of its box centre
// from the node's centre (greedy on the cost -sum_k sign_k(s) * offset_k,
// lowest cost first, ties to the lower child then the lower slot). A ray
// whose direction has sign bits o (bit k set when d_k < 0) then meets the
// children roughly in increasing order of s ^ o, so the traversal orders
// the children it enters with one XOR instead of sorting their distances.
//
// The fold is built in fp32 (8 slots of 32 bytes: (lo.x, lo.y, lo.z, hi.x),
// (hi.y, hi.z, ref, 0), empty slots ref INT_MIN) and then stored quantized,
// 96 bytes per node (k_quantize8, the compression of Ylitie et al. with
// explicit child refs):
//   words 0-2    origin o: the lo corner of the union of the children
//   word 3       int8 exponents ex, ey, ez; the mask of filled slots
//   words 4-15   8-bit child bounds qlo.x[8], qlo.y, qlo.z, qhi.x, qhi.y,
//                qhi.z (slot s in byte s & 3 of word 2 * plane + (s >> 2));
//                an empty slot has qlo = 255, qhi = 0
//   words 16-23  child refs; an empty slot holds ~0 (the leaf of tpre
//                record 0)
// A child's box decodes to o + q * 2^e per axis. qlo is rounded down and
// qhi up, and both are checked against the fp32 box, so the decoded box
// always contains the original one. Refs: >= 0 is an inner child (its node
// number); ~k is a leaf (tpre record k, as in bvh2). An empty slot's
// inverted box misses every ray whose 1/d is not flushed to zero on all
// three axes; should one still pass, its ref sends the lane to test record
// 0, a real triangle, which cannot change a closest hit. The traversal
// therefore needs no filled-mask test per slot.
// Nodes are numbered breadth first, level by level; the inner children of
// one node are consecutive, in slot order.
#include <cuda_runtime.h>

#include <climits>
#include <cstdio>
#include <cstring>

#include "rt_internal.h"

namespace rtgb {

// Quantizes one node: box[s] = (lo.xyz, hi.xyz) of the children in the
// slots of `fmask`, refs copied as given, into the 24 words of a bvh8 node
// (layout above). Per axis the origin is the children's union lo and the
// step the smallest power of two 2^e with extent <= 255 * 2^e; each bound
// becomes a byte, rounded down for lo and up for hi, then checked in fp64
// against the fp32 bound and moved outward if needed, so the decoded box
// o + q * 2^e always contains the original. Empty slots get qlo = 255,
// qhi = 0 and ref ~0. False when some box does not fit the grid (or fmask is
// empty).
__host__ __device__ inline bool quantize_node8(const float box[8][6], const int32_t ref[8], uint32_t fmask,
                                               uint32_t w[24]) {
  fmask &= 0xffu;
  bool ok = fmask != 0;
  if (!ok) fmask = 1;
  for (int i = 0; i < 24; i++) w[i] = 0;
  uint32_t ebytes = fmask << 24;
  for (int k = 0; k < 3; k++) {
    float ulo = 0.0f, uhi = 0.0f;
    bool first = true;
    for (int s = 0; s < 8; s++) {
      if (!((fmask >> s) & 1u)) continue;
      ulo = first ? box[s][k] : fminf(ulo, box[s][k]);
      uhi = first ? box[s][3 + k] : fmaxf(uhi, box[s][3 + k]);
      first = false;
    }
    const double E = (double)uhi - (double)ulo;
    int e = -126;
    if (E > 0.0) {
      int e0 = 0;
      frexp(E / 255.0, &e0);  // E / 255 <= 2^e0
      e = (E <= 255.0 * ldexp(1.0, e0 - 1)) ? e0 - 1 : e0;
      e = e < -126 ? -126 : (e > 127 ? 127 : e);
    }
    const double sc = ldexp(1.0, e);
    if (E > 255.0 * sc) ok = false;
    for (int s = 0; s < 8; s++) {
      int ql = 255, qh = 0;
      if ((fmask >> s) & 1u) {
        const double lo = box[s][k], hi = box[s][3 + k];
        ql = (int)floor((lo - (double)ulo) / sc);
        ql = ql < 0 ? 0 : (ql > 255 ? 255 : ql);
        while (ql > 0 && (double)ulo + ql * sc > lo) ql--;
        qh = (int)ceil((hi - (double)ulo) / sc);
        qh = qh < 0 ? 0 : (qh > 255 ? 255 : qh);
        while (qh < 255 && (double)ulo + qh * sc < hi) qh++;
        if ((double)ulo + ql * sc > lo || (double)ulo + qh * sc < hi) ok = false;
      }
      w[4 + 2 * k + (s >> 2)] |= (uint32_t)ql << (8 * (s & 3));
      w[10 + 2 * k + (s >> 2)] |= (uint32_t)qh << (8 * (s & 3));
    }
    union {
      float f;
      uint32_t u;
    } bits;
    bits.f = ulo;
    w[k] = bits.u;
    ebytes |= ((uint32_t)(e & 0xff)) << (8 * k);
  }
  w[3] = ebytes;
  for (int s = 0; s < 8; s++) w[16 + s] = (fmask >> s) & 1u ? (uint32_t)ref[s] : ~0u;
  return ok;
}

// Octant slot assignment (see the top of this file) of `cnt` child boxes
// (lo.xyz, hi.xyz): slot_of[i] receives child i's slot. Only additions and
// subtractions of the box coordinates are used (twice the centre offsets),
// so host and device give the same assignment.
__host__ __device__ inline void assign_octant_slots(const float (*box)[6], int cnt, int slot_of[8]) {
  float c2[3];
  for (int k = 0; k < 3; k++) {
    float ulo = box[0][k], uhi = box[0][3 + k];
    for (int i = 1; i < cnt; i++) {
      ulo = fminf(ulo, box[i][k]);
      uhi = fmaxf(uhi, box[i][3 + k]);
    }
    c2[k] = ulo + uhi;
  }
  float off[8][3];
  for (int i = 0; i < cnt; i++)
    for (int k = 0; k < 3; k++) off[i][k] = (box[i][k] + box[i][3 + k]) - c2[k];
  uint32_t used_slots = 0, used_kids = 0;
  for (int i = 0; i < 8; i++) slot_of[i] = -1;
  for (int round = 0; round < cnt; round++) {
    float best = 0.0f;
    int bi = -1, bs = -1;
    for (int i = 0; i < cnt; i++) {
      if ((used_kids >> i) & 1u) continue;
      for (int s = 0; s < 8; s++) {
        if ((used_slots >> s) & 1u) continue;
        float cost = 0.0f;
        for (int k = 0; k < 3; k++) cost = ((s >> k) & 1) ? cost - off[i][k] : cost + off[i][k];
        if (bi < 0 || cost < best) {
          best = cost;
          bi = i;
          bs = s;
        }
      }
    }
    slot_of[bi] = bs;
    used_kids |= 1u << bi;
    used_slots |= 1u << bs;
  }
}

namespace {

struct Slot {
  float lo[3], hi[3];
  int32_t ref;
};

__device__ __forceinline__ float slot_area(const Slot &s) {
  float dx = s.hi[0] - s.lo[0], dy = s.hi[1] - s.lo[1], dz = s.hi[2] - s.lo[2];
  return dx * dy + dy * dz + dz * dx;
}

// The two children of bvh2 pair p.
__device__ __forceinline__ void load_pair(const float4 *__restrict__ bvh2, int32_t p, Slot &c0, Slot &c1) {
  const float4 *N = bvh2 + 4ll * p;
  const float4 a = N[0], b = N[1], c = N[2], d = N[3];
  c0.lo[0] = a.x, c0.lo[1] = a.y, c0.hi[0] = a.z, c0.hi[1] = a.w, c0.lo[2] = b.x, c0.hi[2] = b.y;
  c1.lo[0] = c.x, c1.lo[1] = c.y, c1.hi[0] = c.z, c1.hi[1] = c.w, c1.lo[2] = d.x, c1.hi[2] = d.y;
  c0.ref = __float_as_int(b.z);
  c1.ref = __float_as_int(d.z);
}

// ---- SAH collapse: which bvh2 pairs become 8-wide nodes.
// A ray reaches an 8-wide node with probability proportional to the node's
// box area, and every leaf occupies one slot wherever it goes, so the fold
// that minimises the summed area of the chosen nodes minimises the expected
// node visits (the surface area heuristic with fixed leaf cost). Bottom-up
// over the pairs: D(p, j), j = 1..8, is the least summed area for covering
// pair p's subtree with at most j slots, either p itself as one slot (it
// becomes a node: C(p) = area(p) + the best split of 8 slots between its
// children) or its children splitting the j slots; a leaf costs 0. Each
// pair stores D(p, 1..8) and its choices: the split of j slots for j = 2..8
// (0: p stays one slot) and the split of 8 slots when p is a node.

// Parent pair of every inner pair and of every leaf (the root pair: -1).
__global__ void k_pair_parents(const float4 *__restrict__ bvh2, uint32_t n_pairs, int32_t *__restrict__ parent,
                               int32_t *__restrict__ leaf_parent, uint32_t ntris, uint32_t *__restrict__ err) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n_pairs) return;
  const int32_t refs[2] = {__float_as_int(bvh2[4ull * p + 1].z), __float_as_int(bvh2[4ull * p + 3].z)};
  for (int c = 0; c < 2; c++) {
    const int32_t r = refs[c];
    if (r >= 0 ? (uint32_t)r >= n_pairs : (uint32_t)~r >= ntris) {
      atomicOr(err, 1u);
      continue;
    }
    if (r >= 0) parent[r] = (int32_t)p;
    else leaf_parent[~r] = (int32_t)p;
  }
}

// One thread per leaf climbs towards the root; the second thread to reach a
// pair (both children done) computes its costs and climbs on.
__global__ void k_collapse_costs(const float4 *__restrict__ bvh2, uint32_t n_pairs, uint32_t ntris,
                                 const int32_t *__restrict__ parent, const int32_t *__restrict__ leaf_parent,
                                 uint32_t *__restrict__ arrivals, float *__restrict__ cost,
                                 uint32_t *__restrict__ choice, uint32_t *__restrict__ err) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= ntris) return;
  int32_t p = leaf_parent[k];
  for (int climb = 0; p >= 0; climb++) {
    if ((uint32_t)p >= n_pairs || climb > 128) {
      atomicOr(err, 1u);
      return;
    }
    if (atomicAdd(arrivals + p, 1u) == 0u) return;
    __threadfence();
    Slot c[2];
    load_pair(bvh2, p, c[0], c[1]);
    if ((c[0].ref >= 0 && (uint32_t)c[0].ref >= n_pairs) || (c[1].ref >= 0 && (uint32_t)c[1].ref >= n_pairs)) {
      atomicOr(err, 1u);
      return;
    }
    float dc[2][9];
    for (int i = 0; i < 2; i++)
      for (int j = 1; j <= 8; j++) dc[i][j] = c[i].ref >= 0 ? __ldcg(cost + 8ull * c[i].ref + (j - 1)) : 0.0f;
    Slot u = c[0];
    for (int a = 0; a < 3; a++) {
      u.lo[a] = fminf(c[0].lo[a], c[1].lo[a]);
      u.hi[a] = fmaxf(c[0].hi[a], c[1].hi[a]);
    }
    // Best split of j slots between the children, the lower left share first on ties.
    auto split = [&](int j, int &kbest) {
      float best = __int_as_float(0x7f800000);
      kbest = 1;
      for (int l = 1; l < j; l++) {
        const float v = dc[0][l] + dc[1][j - l];
        if (v < best) {
          best = v;
          kbest = l;
        }
      }
      return best;
    };
    int k8;
    const float as_node = slot_area(u) + split(8, k8);
    uint32_t ch = (uint32_t)k8 << 28;
    __stcg(cost + 8ull * p, as_node);
    for (int j = 2; j <= 8; j++) {
      int kj;
      const float v = split(j, kj);
      const bool keep = as_node <= v;
      __stcg(cost + 8ull * p + (j - 1), keep ? as_node : v);
      if (!keep) ch |= (uint32_t)kj << (4 * (j - 2));
    }
    __stcg(choice + p, ch);
    __threadfence();
    p = parent[p];
  }
}

// The SAH choices expanded: pair p0's slots as a node.
__device__ __forceinline__ int sah_slots(const float4 *__restrict__ bvh2, uint32_t n_pairs,
                                         const uint32_t *__restrict__ choice, int32_t p0, Slot (&S)[8],
                                         uint32_t *__restrict__ err) {
  struct Item {
    Slot s;
    int j;
  };
  Item st[8];
  int sp = 0, cnt = 0;
  Slot c0, c1;
  load_pair(bvh2, p0, c0, c1);
  const int k8 = (int)(__ldg(choice + p0) >> 28);
  if (k8 < 1 || k8 > 7) {
    atomicOr(err, 1u);
    return 0;
  }
  st[sp++] = Item{c1, 8 - k8};
  st[sp++] = Item{c0, k8};
  while (sp > 0) {
    const Item it = st[--sp];
    int kj = 0;
    if (it.s.ref >= 0 && it.j >= 2) {
      if ((uint32_t)it.s.ref >= n_pairs) {
        atomicOr(err, 1u);
        return 0;
      }
      kj = (int)((__ldg(choice + it.s.ref) >> (4 * (it.j - 2))) & 15u);
    }
    if (kj == 0) {
      if (cnt >= 8) {
        atomicOr(err, 1u);
        return 0;
      }
      S[cnt++] = it.s;
      continue;
    }
    if (kj >= it.j || sp + 2 > 8) {
      atomicOr(err, 1u);
      return 0;
    }
    load_pair(bvh2, it.s.ref, c0, c1);
    st[sp++] = Item{c1, it.j - kj};
    st[sp++] = Item{c0, kj};
  }
  return cnt;
}

// One frontier node per thread: bvh2 pair frontier[f] becomes bvh8 node
// base + f. inner_cnt[f] receives its number of inner children.
__global__ void k_collapse8(const float4 *__restrict__ bvh2, uint32_t n_pairs, const int32_t *__restrict__ frontier,
                            uint32_t count, uint32_t base, float4 *__restrict__ bvh8, uint32_t *__restrict__ inner_cnt,
                            const uint32_t *__restrict__ choice, uint32_t *__restrict__ err) {
  const uint32_t f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= count) return;
  Slot S[8];
  int cnt = 0;
  const int32_t p0 = frontier[f];
  if (p0 < 0 || (uint32_t)p0 >= n_pairs) {
    atomicOr(err, 1u);
  } else if (choice) {
    cnt = sah_slots(bvh2, n_pairs, choice, p0, S, err);
  } else {
    load_pair(bvh2, p0, S[0], S[1]);
    cnt = 2;
    while (cnt < 8) {
      int pick = -1;
      float best = -1.0f;
      for (int i = 0; i < cnt; i++) {
        if (S[i].ref < 0) continue;
        const float a = slot_area(S[i]);
        if (a > best) {
          best = a;
          pick = i;
        }
      }
      if (pick < 0) break;
      const int32_t p = S[pick].ref;
      if ((uint32_t)p >= n_pairs) {
        atomicOr(err, 1u);
        break;
      }
      load_pair(bvh2, p, S[pick], S[cnt]);
      cnt++;
    }
  }
  float4 *o = bvh8 + 16ull * (base + f);
  const float inf = __int_as_float(0x7f800000);
  for (int s = 0; s < 8; s++) {
    o[2 * s] = make_float4(inf, inf, inf, inf);
    o[2 * s + 1] = make_float4(inf, inf, __int_as_float(INT_MIN), 0.0f);
  }
  uint32_t inner = 0;
  if (cnt > 0) {
    float box[8][6];
    for (int i = 0; i < cnt; i++)
      for (int k = 0; k < 3; k++) {
        box[i][k] = S[i].lo[k];
        box[i][3 + k] = S[i].hi[k];
      }
    int slot_of[8];
    assign_octant_slots(box, cnt, slot_of);
    for (int i = 0; i < cnt; i++) {
      const int s = slot_of[i];
      o[2 * s] = make_float4(S[i].lo[0], S[i].lo[1], S[i].lo[2], S[i].hi[0]);
      o[2 * s + 1] = make_float4(S[i].hi[1], S[i].hi[2], __int_as_float(S[i].ref), 0.0f);
      inner += S[i].ref >= 0 ? 1u : 0u;
    }
  }
  inner_cnt[f] = inner;
}

// Numbers the inner children of the level's nodes (next_base + offs[f] + i)
// and lists their bvh2 pairs as the next frontier.
__global__ void k_link8(uint32_t count, uint32_t base, uint32_t next_base, const uint32_t *__restrict__ offs,
                        float4 *__restrict__ bvh8, int32_t *__restrict__ next_frontier, uint32_t cap,
                        uint32_t *__restrict__ err) {
  const uint32_t f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= count) return;
  float4 *o = bvh8 + 16ull * (base + f);
  uint32_t r = offs[f];
  for (int s = 0; s < 8; s++) {
    float4 w = o[2 * s + 1];
    const int32_t ref = __float_as_int(w.z);
    if (ref < 0) continue;
    if (next_base + r >= cap) {
      atomicOr(err, 2u);
      return;
    }
    next_frontier[r] = ref;
    w.z = __int_as_float((int32_t)(next_base + r));
    o[2 * s + 1] = w;
    r++;
  }
}

// Range-checks every child ref once all levels are built (inner refs
// against the node count, leaf refs against the triangle count); the
// traversal then uses leaf refs without a check.
__global__ void k_encode8(uint32_t n8, uint32_t ntris, const float4 *__restrict__ bvh8, uint32_t *__restrict__ err) {
  const uint32_t f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= n8) return;
  const float4 *o = bvh8 + 16ull * f;
  for (int s = 0; s < 8; s++) {
    const int32_t ref = __float_as_int(o[2 * s + 1].z);
    if (ref == INT_MIN) continue;
    if (ref < 0 ? (uint32_t)~ref >= ntris : (uint32_t)ref >= n8) atomicOr(err, 2u);
  }
}

// fp32 fold -> 96-byte quantized nodes.
__global__ void k_quantize8(const float4 *__restrict__ wide, uint32_t n8, uint4 *__restrict__ out,
                            uint32_t *__restrict__ err) {
  const uint32_t f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= n8) return;
  const float4 *W = wide + 16ull * f;
  float box[8][6];
  int32_t ref[8];
  uint32_t fmask = 0;
  for (int s = 0; s < 8; s++) {
    const float4 a = W[2 * s], b = W[2 * s + 1];
    box[s][0] = a.x, box[s][1] = a.y, box[s][2] = a.z;
    box[s][3] = a.w, box[s][4] = b.x, box[s][5] = b.y;
    ref[s] = __float_as_int(b.z);
    if (ref[s] != INT_MIN) fmask |= 1u << s;
  }
  uint32_t w[24];
  if (!quantize_node8(box, ref, fmask, w)) atomicOr(err, 8u);
  uint4 *o = out + 6ull * f;
  for (int i = 0; i < 6; i++) o[i] = make_uint4(w[4 * i], w[4 * i + 1], w[4 * i + 2], w[4 * i + 3]);
}

}  // namespace

uint32_t bvh8_capacity(uint32_t ntris) { return ntris ? (uint32_t)((4ull * ntris + 6) / 7 + 1) : 0; }

namespace {

// The SAH choices of every pair (k_collapse_costs) into `choice`; `scr`
// holds 10 words per pair plus one per leaf.
cudaError_t collapse_choices(const DevScene &d, uint32_t *scr, uint32_t *choice, uint32_t *errw, cudaStream_t st) {
  const uint32_t n_pairs = d.ntris - 1;
  int32_t *parent = (int32_t *)scr, *leaf_parent = (int32_t *)(scr + n_pairs);
  uint32_t *arrivals = scr + n_pairs + d.ntris;
  float *cost = (float *)(arrivals + n_pairs);
  cudaError_t e = cudaMemsetAsync(parent, 0xff, 4ull * (n_pairs + d.ntris), st);  // parent, leaf_parent: -1
  if (e == cudaSuccess) e = cudaMemsetAsync(arrivals, 0, 4ull * n_pairs, st);
  if (e != cudaSuccess) return e;
  k_pair_parents<<<(n_pairs + 255) / 256, 256, 0, st>>>(d.bvh2, n_pairs, parent, leaf_parent, d.ntris, errw);
  k_collapse_costs<<<(d.ntris + 255) / 256, 256, 0, st>>>(d.bvh2, n_pairs, d.ntris, parent, leaf_parent, arrivals,
                                                          cost, choice, errw);
  return cudaGetLastError();
}

// The fp32 fold (256-byte nodes) into `bvh8`, which holds `cap` nodes:
// pairs chosen by the SAH (sah) or by opening the largest child first.
cudaError_t build_wide_fp32(const DevScene &d, bool sah, float4 *bvh8, uint32_t cap, uint32_t *n8_out,
                            uint32_t *levels_out, int32_t *root_out, char *errbuf, size_t errlen, cudaStream_t st) {
  *n8_out = 0;
  *levels_out = 0;
  *root_out = 0;  // node 0
  if (d.ntris == 0 || cap == 0 || !bvh8) return cudaErrorInvalidValue;
  if (d.root_ref < 0) {
    // One triangle: a single node with the root leaf in slot 0.
    auto bits = [](int32_t i) {
      float f;
      std::memcpy(&f, &i, 4);
      return f;
    };
    float4 h[16];
    const float inf = bits(0x7f800000);
    for (int s = 0; s < 8; s++) {
      h[2 * s] = make_float4(inf, inf, inf, inf);
      h[2 * s + 1] = make_float4(inf, inf, bits(INT_MIN), 0.0f);
    }
    h[0] = make_float4(d.root_lo[0], d.root_lo[1], d.root_lo[2], d.root_hi[0]);
    h[1] = make_float4(d.root_hi[1], d.root_hi[2], bits(d.root_ref), 0.0f);
    cudaError_t e = cudaMemcpyAsync(bvh8, h, sizeof(h), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return e;
    *n8_out = 1;
    *levels_out = 1;
    *root_out = 0;  // node 0: one leaf in slot 0
    return cudaSuccess;
  }
  const uint32_t n_pairs = d.ntris - 1;
  // Scratch: two frontiers, counts, offsets (cap words each), scan sums, error word.
  // With the SAH: the pairs' choices, and for their computation the parent
  // links, arrival counters and costs (11 words per pair, 1 per leaf).
  const size_t sah_words = sah ? 11ull * n_pairs + d.ntris : 0;
  const size_t words = 4ull * cap + cap / 1024 + 8 + sah_words;
  uint32_t *scr = nullptr;
  cudaError_t e = cudaMallocAsync((void **)&scr, 4 * words, st);
  if (e != cudaSuccess) return e;
  int32_t *fr = (int32_t *)scr, *fr_next = (int32_t *)(scr + cap);
  uint32_t *cnt = scr + 2ull * cap, *offs = scr + 3ull * cap, *errw = scr + 4ull * cap;
  uint32_t *sums = errw + 4;
  uint32_t *choice = sah ? sums + cap / 1024 + 4 : nullptr;
  e = cudaMemsetAsync(errw, 0, 4, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(fr, 0, 4, st);  // the root pair is bvh2 record 0
  if (e == cudaSuccess && sah) e = collapse_choices(d, choice + n_pairs, choice, errw, st);
  uint32_t count = 1, base = 0, levels = 0, bad = 0;
  while (e == cudaSuccess && count > 0) {
    if (base + count > cap) {
      bad = 4;
      break;
    }
    const uint32_t grid = (count + 255) / 256;
    k_collapse8<<<grid, 256, 0, st>>>(d.bvh2, n_pairs, fr, count, base, bvh8, cnt, choice, errw);
    e = exclusive_scan_u32(cnt, offs, sums, count, st);
    if (e != cudaSuccess) break;
    k_link8<<<grid, 256, 0, st>>>(count, base, base + count, offs, bvh8, fr_next, cap, errw);
    e = cudaGetLastError();
    uint32_t tail[3] = {0, 0, 0};
    if (e == cudaSuccess) e = cudaMemcpyAsync(&tail[0], offs + count - 1, 4, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&tail[1], cnt + count - 1, 4, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&tail[2], errw, 4, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) break;
    levels++;
    base += count;
    count = tail[0] + tail[1];
    bad = tail[2];
    if (bad) break;
    int32_t *t = fr;
    fr = fr_next;
    fr_next = t;
  }
  if (e == cudaSuccess && !bad) {
    if (base >= (1u << 28)) {
      bad = 4;
    } else {
      k_encode8<<<(base + 255) / 256, 256, 0, st>>>(base, d.ntris, bvh8, errw);
      e = cudaGetLastError();
      uint32_t tail = 0;
      if (e == cudaSuccess) e = cudaMemcpyAsync(&tail, errw, 4, cudaMemcpyDeviceToHost, st);
      if (e == cudaSuccess) e = cudaStreamSynchronize(st);
      bad = tail;
    }
  }
  cudaFreeAsync(scr, st);
  if (e != cudaSuccess) return e;
  if (bad) {
    snprintf(errbuf, errlen, "bvh8 collapse: %s", bad & 4 ? "node capacity exceeded" : "bad child reference");
    return cudaErrorInvalidValue;
  }
  *n8_out = base;
  *levels_out = levels;
  return cudaSuccess;
}

}  // namespace

cudaError_t build_bvh8(const DevScene &d, bool sah, void *bvh8q, uint32_t cap, uint32_t *n8_out,
                       uint32_t *levels_out, int32_t *root_out, char *errbuf, size_t errlen, cudaStream_t st) {
  *n8_out = 0;
  *levels_out = 0;
  if (d.ntris == 0 || cap == 0 || !bvh8q) return cudaErrorInvalidValue;
  float4 *wide = nullptr;
  cudaError_t e = cudaMallocAsync((void **)&wide, 256ull * cap + 256, st);
  if (e != cudaSuccess) return e;
  uint32_t *errw = reinterpret_cast<uint32_t *>(wide + 16ull * cap);
  uint32_t n8 = 0, levels = 0;
  e = build_wide_fp32(d, sah, wide, cap, &n8, &levels, root_out, errbuf, errlen, st);
  // The SAH fold has no node bound below one per pair: past the capacity
  // sized for the largest-first fold, take that fold instead.
  if (e == cudaErrorInvalidValue && sah && strstr(errbuf, "capacity")) {
    errbuf[0] = 0;
    e = build_wide_fp32(d, false, wide, cap, &n8, &levels, root_out, errbuf, errlen, st);
  }
  uint32_t bad = 0;
  if (e == cudaSuccess) e = cudaMemsetAsync(errw, 0, 4, st);
  if (e == cudaSuccess) {
    k_quantize8<<<(n8 + 127) / 128, 128, 0, st>>>(wide, n8, static_cast<uint4 *>(bvh8q), errw);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(&bad, errw, 4, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cudaFreeAsync(wide, st);
  if (e != cudaSuccess) return e;
  if (bad) {
    snprintf(errbuf, errlen, "bvh8: a child box does not fit its node's 8-bit grid");
    return cudaErrorInvalidValue;
  }
  *n8_out = n8;
  *levels_out = levels;
  return cudaSuccess;
}

}  // namespace rtgb

// Host forms of the node quantization and the octant slot assignment, so
// that the containment guarantee and the fold can be checked without a GPU
// (rt_scenes.h).
extern "C" uint32_t rtgbQuantizeNode8(const float *boxes, const int32_t *refs, uint32_t fmask, uint32_t *out) {
  fmask &= 0xffu;
  if (!boxes || !refs || !out || fmask == 0) return 0;
  float box[8][6] = {};
  int32_t ref[8];
  for (uint32_t s = 0; s < 8; s++) {
    const bool f = (fmask >> s) & 1u;
    ref[s] = f ? refs[s] : INT_MIN;
    for (int j = 0; j < 6; j++) box[s][j] = f ? boxes[6 * s + j] : 0.0f;
  }
  return rtgb::quantize_node8(box, ref, fmask, out) ? 1u : 0u;
}

extern "C" uint32_t rtgbAssignOctantSlots(const float *boxes, uint32_t cnt, int32_t *slot_of) {
  if (!boxes || !slot_of || cnt < 1 || cnt > 8) return 0;
  float box[8][6] = {};
  for (uint32_t i = 0; i < cnt; i++)
    for (int j = 0; j < 6; j++) box[i][j] = boxes[6 * i + j];
  int so[8];
  rtgb::assign_octant_slots(box, (int)cnt, so);
  for (uint32_t i = 0; i < cnt; i++) slot_of[i] = so[i];
  return 1;
}
