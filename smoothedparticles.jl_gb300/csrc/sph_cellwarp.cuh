// sph_cellwarp.cuh -- the per-target traversal of the FP64 pair passes (the
// mixed passes in sph_pair32.cu stage candidates the same way but keep hit
// masks; the FP64 density and force passes of a step evaluate each pair once
// in sph_tile64.cu and come here only for rows that overflowed).
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
// Hits are appended, in traversal order, to a per-lane list in global memory
// (see cw_list; the warp's slot of the traversal scratch).  After the
// traversal every lane processes its own list in order, so each target's
// sums are formed in exactly the reference's order, and the lanes' lists
// have nearly equal lengths (the FP64 work runs with full warps).  A list
// that would exceed kTravCap entries is processed early.
#pragma once

#include "sph_common.cuh"
#include "sphgpu.h"

namespace sphgpu {

constexpr int kCwCellBits = 27;             // entry = index | neighbour cell << 27
constexpr int kCwIndexMask = (1 << kCwCellBits) - 1;
constexpr int kCwSkip = -1;

constexpr int kCwBand = 16;  // band candidates a lane may defer

struct CwShared {
  float4 buf[32];             // staged candidates of the current neighbour cell
  float4 offs[27];            // offset of each neighbour cell from the target cell
  int ring[8][32];            // the last < 8 list entries of each lane, column = lane
  short band[kCwBand][32];    // list positions of a lane's unresolved band candidates
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
  return make_float4((float)(qx - t.cx) * k.cellf, (float)(qy - t.cy) * k.cellf,
                     (float)(qz - t.cz) * k.cellf, 0.f);
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

// A lane's list is kTravCap contiguous entries of the warp's slot of the
// traversal scratch (slot < trav_slots; the persistent traversal grid gives
// each warp its own).  Appends go through an 8-entry ring per lane in shared
// memory and reach global memory as whole 32-byte sectors (no partially
// written sectors for the L2 to fill from DRAM); the process phase reads each
// list sequentially.
__device__ __forceinline__ int* cw_list(const BinScratch& b, int slot, int lane) {
  return b.trav + ((size_t)slot * 32 + lane) * kTravCap;
}
constexpr int kCwRow = 1;  // elements between consecutive entries of one list

__device__ __forceinline__ void cw_flush8(const CwShared& sh, int lane, int* dst) {
  const int4 a = make_int4(sh.ring[0][lane], sh.ring[1][lane], sh.ring[2][lane], sh.ring[3][lane]);
  const int4 c = make_int4(sh.ring[4][lane], sh.ring[5][lane], sh.ring[6][lane], sh.ring[7][lane]);
  reinterpret_cast<int4*>(dst)[0] = a;
  reinterpret_cast<int4*>(dst)[1] = c;
}

// writes the ring's pending entries [cnt & ~7, cnt) to the list
__device__ __forceinline__ void cw_flush_tail(const CwShared& sh, int lane, int* list, int cnt) {
  for (int r = cnt & ~7; r < cnt; ++r) list[r] = sh.ring[r & 7][lane];
}

// The reference's FP64 distance test for a candidate in the FP32 band; kept
// out of line so the compiler cannot evaluate it speculatively for every
// candidate.
template <int DIM>
__device__ __noinline__ bool cw_band_test(const State& s, const Consts& k, const double* xp, int q) {
  return within_rn<DIM>(s, k, xp, q);
}

// Band candidates are appended to the list provisionally and tested here, all
// lanes together: on the lattices of the benchmarks many candidates lie
// exactly at r = h (i^2 + j^2 + k^2 = 16 in 3D), and testing each where it is
// found would run the FP64 test one lane at a time.  A rejected candidate's
// entry becomes kCwSkip.
template <int DIM>
__device__ __forceinline__ void cw_resolve(const State& s, const Consts& k, CwShared& sh, int lane,
                                           const CwTarget& t, int* list, int cnt, int& nb) {
  const int kmax = __reduce_max_sync(0xffffffffu, nb);
  for (int kk = 0; kk < kmax; ++kk) {
    if (kk < nb) {
      const int p = sh.band[kk][lane];
      const bool in_ring = p >= (cnt & ~7);
      const int e = in_ring ? sh.ring[p & 7][lane] : list[p];
      if (!within_rn<DIM>(s, k, t.xp, e & kCwIndexMask)) {
        if (in_ring) sh.ring[p & 7][lane] = kCwSkip;
        else list[p] = kCwSkip;
      }
    }
  }
  nb = 0;
}

// P::entry(q, c, type of q) -> the list entry of a hit on q found in
// neighbour cell c, or kCwSkip when the operator ignores it (a skipped hit
// is not an interaction of the operator);
// P::process(list, stride, cnt) consumes cnt entries list[0], list[stride], ...
// skipping kCwSkip entries.  FLUID_CELLS_ONLY: skip neighbour cells without
// fluid (for operators that ignore wall neighbours).
template <int DIM, bool FLUID_CELLS_ONLY, class P>
__device__ __forceinline__ void cw_traverse(const State& s, const Geometry& g, const Consts& k,
                                            const BinScratch& b, CwShared& sh, int lane,
                                            const CwTarget& t, P& proc, int slot) {
  int* const list = cw_list(b, slot, lane);  // dereferenced only by active lanes
  const int cap = kTravCap;
  int cnt = 0;
  int nb = 0;  // deferred band candidates of this lane
  cw_offsets(g, k, sh, lane, t);
  for (int c = 0; c < g.n_diff; ++c) {
    const int nk = t.key + g.key_diff[c];
    if (nk < 1 || nk > g.key_max) continue;  // core.jl:98
    if (FLUID_CELLS_ONLY && __ldg(&b.cell_fluid[nk]) == 0) continue;
    const int st = __ldg(&b.cell_start[nk]);
    const int en = __ldg(&b.cell_start[nk + 1]);
    if (st == en) continue;
    // the target's position relative to this neighbour cell's origin
    const float4 off = sh.offs[c];
    const float ax = t.pi4.x - off.x, ay = t.pi4.y - off.y, az = t.pi4.z - off.z;
    for (int base = st; base < en; base += 32) {
      const int m = min(32, en - base);
      // a chunk adds at most m entries per lane: make room first
      if (__any_sync(0xffffffffu, cnt > cap - m)) {
        cw_resolve<DIM>(s, k, sh, lane, t, list, cnt, nb);
        if (t.active) cw_flush_tail(sh, lane, list, cnt);
        proc.process(list, kCwRow, cnt);
        cnt = 0;
      }
      __syncwarp();
      if (lane < m) sh.buf[lane] = __ldg(&s.pl[base + lane]);
      __syncwarp();
      if (t.active) {
        for (int u0 = 0; u0 < m; u0 += 4) {
          // four candidates' FP32 distances first (independent work), then
          // their hits in candidate order
          float ss4[4];
          int tq4[4];
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            const float4 pq = sh.buf[min(u0 + j, 31)];
            const float dx = ax - pq.x;
            const float dy = ay - pq.y;
            float ss = dx * dx + dy * dy;
            if (DIM == 3) {
              const float dz = az - pq.z;
              ss = ss + dz * dz;
            }
            ss4[j] = ss;
            tq4[j] = __float_as_int(pq.w);
          }
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            const int q = base + u0 + j;
            if (u0 + j < m && !(ss4[j] > k.s_hi) && q != t.i) {
              int e = proc.entry(q, c, tq4[j]);
              if (e != kCwSkip && !(ss4[j] < k.s_lo)) {
                // in the band: defer the FP64 test, or take it now when this
                // lane's deferral slots are full
                if (nb < kCwBand) {
                  sh.band[nb][lane] = (short)cnt;
                  ++nb;
                } else if (!cw_band_test<DIM>(s, k, t.xp, q)) {
                  e = kCwSkip;
                }
              }
              if (e != kCwSkip) {
                sh.ring[cnt & 7][lane] = e;
                ++cnt;
                if ((cnt & 7) == 0) cw_flush8(sh, lane, list + (cnt - 8));
              }
            }
          }
        }
      }
    }
  }
  cw_resolve<DIM>(s, k, sh, lane, t, list, cnt, nb);
  if (t.active) cw_flush_tail(sh, lane, list, cnt);
  __syncwarp();
  proc.process(list, kCwRow, cnt);
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
// Pair interactions = every processed entry.
template <int OP>
__device__ __forceinline__ void cw_count(const BinScratch& b, int c0, int c1, int c2) {
  cw_warp_add(b.d_pairs, c0 + c1);
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

// The pair passes' common skeleton: the traversal of the warp's item (the
// density and force passes of a step sum rows instead, sph_pair64.cu, and
// come here only for targets whose rows overflowed).
template <int DIM, int OP, class P>
__device__ __forceinline__ void cw_pass(const State& s, const Geometry& g, const Consts& k,
                                        const BinScratch& b, CwShared& sh, int lane,
                                        const CwTarget& t, P& proc, int slot) {
  cw_traverse<DIM, OP == SPH_OP_WALL_PRESSURE>(s, g, k, b, sh, lane, t, proc, slot);
}

// d = x_p - x_q and the kernel distance sqrt((d0 d0 + d1 d1) + d2 d2) with the
// sum fused (the support test, within_rn, keeps the reference's unfused form)
template <int DIM>
__device__ __forceinline__ double kdist64(const State& s, const double* xp, int q, double* d) {
  d[0] = xp[0] - __ldg(&s.x[0][q]);
  d[1] = xp[1] - __ldg(&s.x[1][q]);
  double ss = __fma_rn(d[1], d[1], d[0] * d[0]);
  if (DIM == 3) {
    d[2] = xp[2] - __ldg(&s.x[2][q]);
    ss = __fma_rn(d[2], d[2], ss);
  } else {
    d[2] = 0.0;
  }
  return sqrt(ss);
}

}  // namespace sphgpu
