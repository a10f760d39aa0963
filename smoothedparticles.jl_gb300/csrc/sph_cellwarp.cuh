// sph_cellwarp.cuh -- the traversal shared by the FP64 and mixed pair passes.
//
// One warp per work item: up to 32 targets of ONE cell (the work list is built
// with the binning).  All lanes share the cell, so they share the neighbour
// sequence of _apply_binary! (core.jl:96-103): the neighbour cells in key_diff
// order, each cell's particles in stored (descending reference index) order.
// For every neighbour cell the warp
//   * computes the cell's offset from the target cell once (uniform),
//   * stages the cell's particles 32 at a time into shared memory with one
//     coalesced 512-byte load (cell-relative FP32 position + type),
//   * lets every lane test every staged candidate through broadcast reads.
// A candidate is classified in FP32; only candidates within a thin band around
// the support radius take the reference's FP64 test (proof in sph_pair64.cu).
//
// Hits are appended, in traversal order, to the target's column of the hit
// list in global memory (entry t of target i at hits[t * stride + i]; the
// warp's 32 consecutive targets make each append one coalesced 128-byte
// row).  After the traversal every lane processes its own list in order, so
// each target's sums are formed in exactly the reference's order, and the
// lanes' lists have nearly equal lengths (the FP64 work runs with full
// warps).  The force pass of the same binning reads the lists back instead of
// traversing again.  A list that would exceed hit_cap is processed early and
// its item is marked partial (the force pass then traverses that item).
#pragma once

#include "sph_common.cuh"
#include "sphgpu.h"

namespace sphgpu {

constexpr int kCwWarps = 4;                 // warps per block
constexpr int kCwThreads = 32 * kCwWarps;
constexpr int kCwCellBits = 27;             // entry = index | neighbour cell << 27
constexpr int kCwIndexMask = (1 << kCwCellBits) - 1;
constexpr int kCwSkip = -1;

struct CwShared {
  float4 buf[32];      // staged candidates of the current neighbour cell
  float4 offs[27];     // offset of each neighbour cell from the target cell
};

struct CwTarget {
  bool active;         // lane holds a target the operator acts on
  int i;               // target index (sorted order)
  int key, cx, cy, cz; // target cell
  float4 pi4;          // cell-relative FP32 position
  double xp[3];        // FP64 position (band test)
};

__device__ __forceinline__ float4 cw_offset(const Geometry& g, const Consts& k, const CwTarget& t,
                                            int nk) {
  int qx, qy, qz;
  decode_key(g, nk, qx, qy, qz);
  return make_float4((float)(qx - t.cx) * k.hf, (float)(qy - t.cy) * k.hf,
                     (float)(qz - t.cz) * k.hf, 0.f);
}

// Fills sh.offs for every neighbour cell (lanes 0..n_diff-1, one each).
__device__ __forceinline__ void cw_offsets(const Geometry& g, const Consts& k, CwShared& sh,
                                           int lane, const CwTarget& t) {
  if (lane < g.n_diff) {
    const int nk = t.key + g.key_diff[lane];
    sh.offs[lane] = (nk >= 1 && nk <= g.key_max) ? cw_offset(g, k, t, nk)
                                                 : make_float4(0.f, 0.f, 0.f, 0.f);
  }
  __syncwarp();
}

// P::entry(q, c, type of q) -> the list entry of a hit on q found in
// neighbour cell c, or kCwSkip when the operator ignores it;
// P::process(list, stride, cnt) consumes cnt entries list[0], list[stride], ...
// Returns the number of entries left in the list; sets `partial` when the
// list was processed early.
template <int DIM, class P>
__device__ __forceinline__ int cw_traverse(const State& s, const Geometry& g, const Consts& k,
                                           const BinScratch& b, CwShared& sh, int lane,
                                           const CwTarget& t, P& proc, int& pairs,
                                           bool& partial) {
  int* const list = b.hits + t.i;  // dereferenced only by active lanes
  const int stride = b.hit_stride;
  const int cap = b.hit_cap;
  int cnt = 0;
  cw_offsets(g, k, sh, lane, t);
  for (int c = 0; c < g.n_diff; ++c) {
    const int nk = t.key + g.key_diff[c];
    if (nk < 1 || nk > g.key_max) continue;  // core.jl:98
    const int st = __ldg(&b.cell_start[nk]);
    const int en = __ldg(&b.cell_start[nk + 1]);
    if (st == en) continue;
    const float4 off = sh.offs[c];
    for (int base = st; base < en; base += 32) {
      const int m = min(32, en - base);
      __syncwarp();
      if (lane < m) sh.buf[lane] = __ldg(&s.pl[base + lane]);
      __syncwarp();
      for (int u = 0; u < m; ++u) {
        const float4 pq = sh.buf[u];
        if (t.active) {
          const int q = base + u;
          const float dx = (t.pi4.x - pq.x) - off.x;
          const float dy = (t.pi4.y - pq.y) - off.y;
          float ss = dx * dx + dy * dy;
          if (DIM == 3) {
            const float dz = (t.pi4.z - pq.z) - off.z;
            ss = ss + dz * dz;
          }
          if (!(ss > k.s_hi) && q != t.i && (ss < k.s_lo || within_rn<DIM>(s, k, t.xp, q))) {
            ++pairs;
            const int e = proc.entry(q, c, __float_as_int(pq.w));
            if (e != kCwSkip) {
              list[(size_t)cnt * stride] = e;
              ++cnt;
            }
          }
        }
        if (__any_sync(0xffffffffu, cnt == cap)) {
          proc.process(list, stride, cnt);
          cnt = 0;
          partial = true;
        }
      }
    }
  }
  __syncwarp();
  proc.process(list, stride, cnt);
  return cnt;
}

// Loads the warp's work item.  Returns false when the warp has no item.
__device__ __forceinline__ bool cw_item(const BinScratch& b, const Geometry& g, int warp_global,
                                        int& first, int& count) {
  const int total = __ldg(&b.item_off[g.key_max + 1]);
  if (warp_global >= total) return false;
  const int2 it = __ldg(&b.items[warp_global]);
  first = it.x;
  count = it.y;
  return true;
}

__device__ __forceinline__ void cw_warp_add(unsigned long long* dst, int v) {
  const int sum = __reduce_add_sync(0xffffffffu, v);
  if ((threadIdx.x & 31) == 0 && sum) atomicAdd(dst, (unsigned long long)sum);
}

// Pair and per-category hit counters (c0: the operator's main hits; for the
// force c0 = fluid neighbours, c1 = wall neighbours, c2 = viscosity active).
template <int OP>
__device__ __forceinline__ void cw_count(const BinScratch& b, int pairs, int c0, int c1, int c2) {
  cw_warp_add(b.d_pairs, pairs);
  if (OP == SPH_OP_FORCE) {
    cw_warp_add(b.d_cat + kCatForceFluid, c0);
    cw_warp_add(b.d_cat + kCatForceWall, c1);
    cw_warp_add(b.d_cat + kCatForceAV, c2);
  } else if (OP == SPH_OP_WALL_PRESSURE) {
    cw_warp_add(b.d_cat + kCatWall, c0);
  } else {
    cw_warp_add(b.d_cat + kCatDensity, c0);
  }
}

// The pair passes' common skeleton.  list_mode: 0 traverse only, 1 traverse
// and keep the lists (density passes), 2 read the lists kept by the density
// pass of this binning (force pass; partial items traverse).
template <int DIM, int OP, class P>
__device__ __forceinline__ void cw_pass(const State& s, const Geometry& g, const Consts& k,
                                        const BinScratch& b, CwShared& sh, int lane, int item,
                                        const CwTarget& t, P& proc, int& pairs, int list_mode) {
  if (list_mode == 2 && __ldg(&b.item_partial[item]) == 0) {
    cw_offsets(g, k, sh, lane, t);
    if (t.active) {
      const int cnt = __ldg(&b.hit_count[t.i]);
      pairs += cnt;
      proc.process(b.hits + t.i, b.hit_stride, cnt);
    }
    __syncwarp();
    return;
  }
  bool partial = false;
  const int left = cw_traverse<DIM>(s, g, k, b, sh, lane, t, proc, pairs, partial);
  if (list_mode == 1) {
    if (t.active) b.hit_count[t.i] = left;
    if (lane == 0) b.item_partial[item] = partial ? 1 : 0;
  }
}

}  // namespace sphgpu
