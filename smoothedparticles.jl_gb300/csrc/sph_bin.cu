// sph_bin.cu -- create_cell_list! (core.jl:51-90) as a counting sort by cell key.
//
// Per binning (all HBM-bound, one thread per particle unless noted):
//   1. bin_keys     : [step: kick + drift] removal test against the domain's
//                     bounding box, 1-based linear cell key (structs.jl:97-106),
//                     bucket slot by a warp-aggregated atomicAdd on the cell's
//                     count.  Removed particles get key key_max+1.
//   2. bin_remove   : one CTA; no-op unless something was removed.  Replays the
//                     reference's tail-fill compaction (core.jl:71-81) on
//                     reference indices only, so survivors get the index the
//                     reference would give them.
//   3. scan         : exclusive prefix sum of the key_max+3 counts -> cell starts
//                     (a counting sort is the one-digit radix sort whose radix
//                     is the number of cells).
//   4. bin_scatter  : bucket position = cell start + slot.
//   5. bin_rank     : one warp per cell; orders the bucket by DESCENDING
//                     reference index, which is the order add_index! keeps
//                     (core.jl:26-41) and the order the pair loop sums in.
//   6. bin_gather   : reorders the SoA into the new slots, writes the cell key,
//                     the FP32 cell-relative position and the inverse index map,
//                     and publishes the new particle count.
#include "sph_launch.h"
#include "sphgpu.h"

namespace sphgpu {

namespace {

constexpr int kThreads = 256;

template <int DIM>
__device__ __forceinline__ void bin_keys_body(const State& s, const Geometry& g, const Consts& k, const BinScratch& b, int step_mode, int blk) {
  const int n = *b.d_n;
  const int i = blk * kThreads + threadIdx.x;
  if (i >= n) return;
  double x[3];
  x[0] = s.x[0][i];
  x[1] = s.x[1][i];
  x[2] = DIM == 3 ? s.x[2][i] : 0.0;
  if (step_mode && s.type[i] == kFluid) {
    // accelerate! then move! (collapse_symplectic.jl:133-143), per component
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
      const double vd = s.v[d][i] + k.hdt * (s.a[d][i] + k.g[d]);
      s.v[d][i] = vd;
      x[d] = x[d] + k.dt * (vd + k.eps_xsph * s.xs[d][i]);
      s.x[d][i] = x[d];
    }
  }
  bool inside = true;  // geometry.jl:24-30; false for NaN
#pragma unroll
  for (int d = 0; d < 3; ++d) inside = inside && (k.dmin[d] <= x[d]) && (x[d] <= k.dmax[d]);
  int key;
  if (!inside) {
    key = g.key_max + 1;
    b.flag_by_rid[s.rid[i]] = 1;
    atomicAdd(b.d_nrem, 1);
  } else {
    long long ijk[3];
#pragma unroll
    for (int d = 0; d < 3; ++d)
      ijk[d] = 1 + (long long)floor(cell_coord(k, x[d], d)) - g.key_phase[d];
    const long long kk =
        ijk[0] + g.key_lim[0] * (ijk[1] - 1) + g.key_lim[0] * g.key_lim[1] * (ijk[2] - 1);
    if (kk < 1 || kk > g.key_max) {  // cannot happen for a point inside the box
      atomicOr(b.d_err, kErrKeyRange);
      key = g.key_max + 1;
      b.flag_by_rid[s.rid[i]] = 1;
      atomicAdd(b.d_nrem, 1);
    } else {
      key = (int)kk;
    }
  }
  b.keys[i] = key;
  // warp-aggregated bucket slot: one atomic per distinct key in the warp
  const unsigned active = __activemask();
  const unsigned peers = __match_any_sync(active, key);
  const int leader = __ffs(peers) - 1;
  const int lane = threadIdx.x & 31;
  int base = 0;
  if (lane == leader) base = atomicAdd(&b.counts[key], __popc(peers));
  base = __shfl_sync(peers, base, leader);
  b.slots[i] = base + __popc(peers & lanemask_lt());
}

template <int DIM>
__global__ void __launch_bounds__(kThreads) bin_keys_kernel(State s, Geometry g, Consts k,
                                                            BinScratch b, int step_mode) {
  bin_keys_body<DIM>(s, g, k, b, step_mode, blockIdx.x);
}

// Block-wide exclusive scan of one int per thread (blockDim.x == 1024 or a
// multiple of 32); returns the exclusive prefix, *total gets the block sum.
__device__ __forceinline__ int block_exclusive_scan(int v, int* warp_sums, int* total) {
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int nwarps = blockDim.x >> 5;
  int incl = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += t;
  }
  if (lane == 31) warp_sums[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    int w = lane < nwarps ? warp_sums[lane] : 0;
    int wi = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(0xffffffffu, wi, o);
      if (lane >= o) wi += t;
    }
    if (lane < nwarps) warp_sums[lane] = wi - w;
    if (lane == 31) warp_sums[32] = wi;
  }
  __syncthreads();
  const int excl = warp_sums[warp] + incl - v;
  *total = warp_sums[32];
  __syncthreads();
  return excl;
}

// core.jl:71-81 replayed on reference indices (one CTA of 1024 threads).
__device__ __forceinline__ void bin_remove_body(const BinScratch& b, int blk) {
  const int k = *b.d_nrem;
  if (k == 0) return;
  const int N = *b.d_n;
  __shared__ int warp_sums[33];
  int carry = 0;
  // removed reference indices in ascending order
  for (int base = 0; base < N; base += blockDim.x) {
    const int idx = base + threadIdx.x;
    const int f = idx < N ? b.flag_by_rid[idx] : 0;
    int total;
    const int excl = block_exclusive_scan(f, warp_sums, &total);
    if (f) {
      b.rem_list[carry + excl] = idx;
      b.flag_by_rid[idx] = 0;
    }
    carry += total;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    // particles[removal[t]] = particles[end+1-t] for the removal entries in
    // descending order; ident[p] tracks which reference index sits at p.
    for (int t = 0; t < k; ++t) {
      const int r = b.rem_list[k - 1 - t];
      const int last = N - 1 - t;
      b.ident[r] = b.ident[last];
    }
    for (int t = 0; t < k; ++t) {
      const int r = b.rem_list[t];
      if (r < N - k) b.moved_to[b.ident[r]] = r;
    }
    for (int t = 0; t < k; ++t) b.ident[b.rem_list[t]] = b.rem_list[t];
  }
}

__global__ void __launch_bounds__(1024) bin_remove_kernel(BinScratch b) {
  bin_remove_body(b, blockIdx.x);
}

__device__ __forceinline__ void bin_scatter_body(const State& s, const Geometry& g, const BinScratch& b, int blk) {
  const int n = *b.d_n;
  const int i = blk * kThreads + threadIdx.x;
  if (i >= n) return;
  const int key = b.keys[i];
  const int dst = b.cell_start[key] + b.slots[i];
  b.perm_tmp[dst] = i;
  int rid = s.rid[i];
  const int nrem = *b.d_nrem;
  if (nrem > 0 && key <= g.key_max && rid >= n - nrem) rid = b.moved_to[rid];
  b.rid_tmp[dst] = rid;
}

__global__ void __launch_bounds__(kThreads) bin_scatter_kernel(State s, Geometry g, BinScratch b) {
  bin_scatter_body(s, g, b, blockIdx.x);
}

// One warp per cell: slot of element e = number of elements of the cell with
// a larger reference index (reference indices are unique).
__device__ __forceinline__ void bin_rank_body(const Geometry& g, const BinScratch& b, int blk) {
  const int lane = threadIdx.x & 31;
  const int cell = blk * (kThreads / 32) + (threadIdx.x >> 5) + 1;
  if (cell > g.key_max) return;
  const int st = b.cell_start[cell];
  const int en = b.cell_start[cell + 1];
  const int cnt = en - st;
  if (cnt == 0) return;
  if (cnt <= 32) {
    const int my = lane < cnt ? b.rid_tmp[st + lane] : -1;
    const int pm = lane < cnt ? b.perm_tmp[st + lane] : 0;
    int rank = 0;
    for (int f = 0; f < cnt; ++f) rank += (__shfl_sync(0xffffffffu, my, f) > my);
    if (lane < cnt) {
      b.perm[st + rank] = pm;
      b.rid_sorted[st + rank] = my;
    }
    return;
  }
  for (int e = st + lane; e < en; e += 32) {
    const int my = b.rid_tmp[e];
    int rank = 0;
    for (int f = st; f < en; ++f) rank += (b.rid_tmp[f] > my);
    b.perm[st + rank] = b.perm_tmp[e];
    b.rid_sorted[st + rank] = my;
  }
}

__global__ void __launch_bounds__(kThreads) bin_rank_kernel(Geometry g, BinScratch b) {
  bin_rank_body(g, b, blockIdx.x);
}

template <int DIM>
__device__ __forceinline__ void bin_gather_body(const State& cur, const State& alt, const Geometry& g, const Consts& k, const BinScratch& b, int gather_all, int blk) {
  const int n_new = b.cell_start[g.key_max + 1];
  const int dst = blk * kThreads + threadIdx.x;
  if (dst == 0) *b.d_n = n_new;
  if (dst >= n_new) return;
  const int src = b.perm[dst];
  const int key = b.keys[src];
  const int rid = b.rid_sorted[dst];
  int cx, cy, cz;
  decode_key(g, key, cx, cy, cz);
  const int cc[3] = {cx, cy, cz};
  float xl[3] = {0.f, 0.f, 0.f};
#pragma unroll
  for (int d = 0; d < DIM; ++d) {
    const double xd = cur.x[d][src];
    alt.x[d][dst] = xd;
    alt.v[d][dst] = cur.v[d][src];
    const double origin = (double)(g.key_phase[d] + cc[d]) * k.cell + k.shift[d];
    xl[d] = (float)(xd - origin);
    if (gather_all) {
      alt.a[d][dst] = cur.a[d][src];
      alt.xs[d][dst] = cur.xs[d][src];
    }
  }
  const int t = cur.type[src];
  alt.rho_ref[dst] = cur.rho_ref[src];
  alt.type[dst] = t;
  alt.oid[dst] = cur.oid[src];
  alt.rid[dst] = rid;
  alt.cell[dst] = key;
  alt.pl[dst] = make_float4(xl[0], xl[1], xl[2], __int_as_float(t));
  // mixed precision: the position half of the FP32 neighbour record, with the
  // type in the sign bit (the pair passes fill in rho, v and P/rho^2)
  if (alt.rec) alt.rec[2 * dst] = make_float4(xl[0], xl[1], xl[2], t == kFluid ? 1.f : -1.f);
  b.inv_rid[rid] = dst;
  if (t == kFluid) {  // fluid per cell, one atomic per cell and warp
    const unsigned peers = __match_any_sync(__activemask(), key);
    if ((int)(threadIdx.x & 31) == __ffs(peers) - 1) atomicAdd(&b.cell_fluid[key], __popc(peers));
  }
  if (gather_all) {
    alt.rho[dst] = cur.rho[src];
    alt.P[dst] = cur.P[src];
    alt.Pr[dst] = cur.Pr[src];
  }
}

template <int DIM>
__global__ void __launch_bounds__(kThreads) bin_gather_kernel(State cur, State alt, Geometry g,
                                                              Consts k, BinScratch b,
                                                              int gather_all) {
  bin_gather_body<DIM>(cur, alt, g, k, b, gather_all, blockIdx.x);
}

// ---- pair-pass work list: cell k gets ceil(c_k / 32) items of <= 32 targets
__device__ __forceinline__ void items_count_body(const Geometry& g, const BinScratch& b, int blk) {
  const int k = blk * kThreads + threadIdx.x;  // 0 .. key_max + 2
  if (k > g.key_max + 2) return;
  int c = 0;
  if (k >= 1 && k <= g.key_max) c = (b.cell_start[k + 1] - b.cell_start[k] + 31) >> 5;
  b.counts[k] = c;  // the bucket counts are no longer needed once the starts exist
}

__global__ void __launch_bounds__(kThreads) items_count_kernel(Geometry g, BinScratch b) {
  items_count_body(g, b, blockIdx.x);
}

__device__ __forceinline__ void items_write_body(const Geometry& g, const BinScratch& b, int blk) {
  const int k = blk * kThreads + threadIdx.x + 1;
  if (k > g.key_max) return;
  const int st = b.cell_start[k];
  const int c = b.cell_start[k + 1] - st;
  int off = b.item_off[k];
  for (int t = 0; t < c; t += 32, ++off) b.items[off] = make_int2(st + t, min(32, c - t));
}

__global__ void __launch_bounds__(kThreads) items_write_kernel(Geometry g, BinScratch b) {
  items_write_body(g, b, blockIdx.x);
}

// ---- mask slots of the mixed-precision pair passes: every item of a cell
// with fluid gets one slot per 32-candidate chunk of the cell's neighbour
// cells (the chunk sequence of the pair traversal)
__device__ __forceinline__ void chunks_count_body(const Geometry& g, const BinScratch& b, int blk) {
  const int k = blk * kThreads + threadIdx.x;  // 0 .. key_max + 2
  if (k > g.key_max + 2) return;
  int v = 0;
  if (k >= 1 && k <= g.key_max && b.cell_fluid[k] > 0) {
    int nc = 0;
    for (int j = 0; j < g.n_diff; ++j) {
      const int nk = k + g.key_diff[j];
      if (nk >= 1 && nk <= g.key_max) nc += (b.cell_start[nk + 1] - b.cell_start[nk] + 31) >> 5;
    }
    v = ((b.cell_start[k + 1] - b.cell_start[k] + 31) >> 5) * nc;
  }
  b.counts[k] = v;  // the item counts are no longer needed once items exist
}

__global__ void __launch_bounds__(kThreads) chunks_count_kernel(Geometry g, BinScratch b) {
  chunks_count_body(g, b, blockIdx.x);
}

// ---- generic exclusive scan (3 kernels)
constexpr int kScanThreads = 512;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;

__device__ __forceinline__ void scan_reduce_body(const int* in, int len, int* tmp, int blk) {
  __shared__ int warp_sums[33];
  const int base = blk * kScanTile;
  int v = 0;
#pragma unroll
  for (int t = 0; t < kScanItems; ++t) {
    const int idx = base + t * kScanThreads + threadIdx.x;
    if (idx < len) v += in[idx];
  }
  int total;
  block_exclusive_scan(v, warp_sums, &total);
  if (threadIdx.x == 0) tmp[blk] = total;
}

__global__ void __launch_bounds__(kScanThreads) scan_reduce_kernel(const int* in, int len, int* tmp) {
  scan_reduce_body(in, len, tmp, blockIdx.x);
}

__device__ __forceinline__ void scan_blocks_body(int* tmp, int nblocks, int blk) {
  __shared__ int warp_sums[33];
  int carry = 0;
  for (int base = 0; base < nblocks; base += blockDim.x) {
    const int idx = base + threadIdx.x;
    const int v = idx < nblocks ? tmp[idx] : 0;
    int total;
    const int excl = block_exclusive_scan(v, warp_sums, &total);
    if (idx < nblocks) tmp[idx] = carry + excl;
    carry += total;
  }
}

__global__ void __launch_bounds__(1024) scan_blocks_kernel(int* tmp, int nblocks) {
  scan_blocks_body(tmp, nblocks, blockIdx.x);
}

__device__ __forceinline__ void scan_apply_body(const int* in, int* out, int len, const int* tmp, int blk) {
  __shared__ int warp_sums[33];
  const int base = blk * kScanTile + threadIdx.x * kScanItems;
  int vals[kScanItems];
  int sum = 0;
#pragma unroll
  for (int t = 0; t < kScanItems; ++t) {
    const int idx = base + t;
    vals[t] = idx < len ? in[idx] : 0;
    sum += vals[t];
  }
  int total;
  int run = block_exclusive_scan(sum, warp_sums, &total) + tmp[blk];
#pragma unroll
  for (int t = 0; t < kScanItems; ++t) {
    const int idx = base + t;
    if (idx < len) out[idx] = run;
    run += vals[t];
  }
}

__global__ void __launch_bounds__(kScanThreads) scan_apply_kernel(const int* in, int* out, int len,
                                                                  const int* tmp) {
  scan_apply_body(in, out, len, tmp, blockIdx.x);
}

// ---- fused batches: the same bodies, one launch over all members; block i
// of a shape works on map[i] = (member, block of that member)
struct FusedArgs {
  const MemberArgs* __restrict__ m;
  const int2* __restrict__ map;
};

__device__ __forceinline__ const MemberArgs& fused_member(const FusedArgs& f, int2& e) {
  e = f.map[blockIdx.x];
  return f.m[e.x];
}

__global__ void __launch_bounds__(kThreads) fused_clear_kernel(FusedArgs f) {
  int2 e;
  const MemberArgs& m = fused_member(f, e);
  const int k = e.y * kThreads + threadIdx.x;
  if (k < m.g.key_max + 3) {
    m.b.counts[k] = 0;
    m.b.cell_fluid[k] = 0;
  }
  if (e.y == 0 && threadIdx.x == 0) *m.b.d_nrem = 0;
}

template <int DIM>
__global__ void __launch_bounds__(kThreads) fused_keys_kernel(FusedArgs f) {
  int2 e;
  const MemberArgs& m = fused_member(f, e);
  bin_keys_body<DIM>(m.cur, m.g, m.k, m.b, 1, e.y);
}

__global__ void __launch_bounds__(1024) fused_remove_kernel(FusedArgs f) {
  int2 e;
  const MemberArgs& m = fused_member(f, e);
  bin_remove_body(m.b, e.y);
}

// which: 0 counts -> cell_start, 1 counts -> item_off, 2 counts -> chunk_off
__device__ __forceinline__ int* fused_scan_out(const MemberArgs& m, int which) {
  return which == 0 ? m.b.cell_start : which == 1 ? m.b.item_off : m.b.chunk_off;
}

__global__ void __launch_bounds__(kScanThreads) fused_scan_reduce_kernel(FusedArgs f) {
  int2 e;
  const MemberArgs& m = fused_member(f, e);
  scan_reduce_body(m.b.counts, m.g.key_max + 3, m.b.scan_tmp, e.y);
}

__global__ void __launch_bounds__(1024) fused_scan_blocks_kernel(FusedArgs f) {
  int2 e;
  const MemberArgs& m = fused_member(f, e);
  scan_blocks_body(m.b.scan_tmp, (m.g.key_max + 3 + kScanTile - 1) / kScanTile, e.y);
}

__global__ void __launch_bounds__(kScanThreads) fused_scan_apply_kernel(FusedArgs f, int which) {
  int2 e;
  const MemberArgs& m = fused_member(f, e);
  scan_apply_body(m.b.counts, fused_scan_out(m, which), m.g.key_max + 3, m.b.scan_tmp, e.y);
}

__global__ void __launch_bounds__(kThreads) fused_scatter_kernel(FusedArgs f) {
  int2 e;
  const MemberArgs& m = fused_member(f, e);
  bin_scatter_body(m.cur, m.g, m.b, e.y);
}

__global__ void __launch_bounds__(kThreads) fused_rank_kernel(FusedArgs f) {
  int2 e;
  const MemberArgs& m = fused_member(f, e);
  bin_rank_body(m.g, m.b, e.y);
}

__global__ void __launch_bounds__(kThreads) fused_items_count_kernel(FusedArgs f) {
  int2 e;
  const MemberArgs& m = fused_member(f, e);
  items_count_body(m.g, m.b, e.y);
}

__global__ void __launch_bounds__(kThreads) fused_items_write_kernel(FusedArgs f) {
  int2 e;
  const MemberArgs& m = fused_member(f, e);
  items_write_body(m.g, m.b, e.y);
}

template <int DIM>
__global__ void __launch_bounds__(kThreads) fused_gather_kernel(FusedArgs f) {
  int2 e;
  const MemberArgs& m = fused_member(f, e);
  bin_gather_body<DIM>(m.cur, m.alt, m.g, m.k, m.b, kGatherStep, e.y);
}

__global__ void __launch_bounds__(kThreads) fused_chunks_count_kernel(FusedArgs f) {
  int2 e;
  const MemberArgs& m = fused_member(f, e);
  chunks_count_body(m.g, m.b, e.y);
}

}  // namespace

int fused_blocks(int shape, int cap, int key_max, int max_items, int warps) {
  const int nb = key_max + 3;
  switch (shape) {
    case kShapeParticles: return (cap + kThreads - 1) / kThreads;
    case kShapeBuckets: return (nb + kThreads - 1) / kThreads;
    case kShapeCells: return (key_max + kThreads - 1) / kThreads;
    case kShapeRank: return (key_max + (kThreads / 32) - 1) / (kThreads / 32);
    case kShapeScanTiles: return (nb + kScanTile - 1) / kScanTile;
    case kShapeMember: return 1;
    case kShapeItems: return (max_items + warps - 1) / warps;
    default: return 0;
  }
}

// The binning of one fused step (launch_binning for every member): members'
// state args[p].cur -> args[p].alt.
cudaError_t launch_fused_binning(const LaunchCtx& c, const FusedBatch& fb, int p) {
  auto fa = [&](int shape) { return FusedArgs{fb.args[p], fb.map[shape]}; };
  auto grid = [&](int shape) { return (unsigned)fb.blocks[shape]; };
  cudaStream_t st = c.stream;
  mark(c, SPH_KERNEL_BIN_KEYS, 0);
  fused_clear_kernel<<<grid(kShapeBuckets), kThreads, 0, st>>>(fa(kShapeBuckets));
  if (fb.dim == 2)
    fused_keys_kernel<2><<<grid(kShapeParticles), kThreads, 0, st>>>(fa(kShapeParticles));
  else
    fused_keys_kernel<3><<<grid(kShapeParticles), kThreads, 0, st>>>(fa(kShapeParticles));
  mark(c, SPH_KERNEL_BIN_KEYS, 1, 2);
  mark(c, SPH_KERNEL_BIN_REMOVE, 0);
  fused_remove_kernel<<<grid(kShapeMember), 1024, 0, st>>>(fa(kShapeMember));
  mark(c, SPH_KERNEL_BIN_REMOVE, 1);
  auto scan = [&](int which) {
    mark(c, SPH_KERNEL_BIN_SCAN, 0);
    fused_scan_reduce_kernel<<<grid(kShapeScanTiles), kScanThreads, 0, st>>>(fa(kShapeScanTiles));
    fused_scan_blocks_kernel<<<grid(kShapeMember), 1024, 0, st>>>(fa(kShapeMember));
    fused_scan_apply_kernel<<<grid(kShapeScanTiles), kScanThreads, 0, st>>>(fa(kShapeScanTiles),
                                                                             which);
    mark(c, SPH_KERNEL_BIN_SCAN, 1, 3);
  };
  scan(0);
  mark(c, SPH_KERNEL_BIN_SCATTER, 0);
  fused_scatter_kernel<<<grid(kShapeParticles), kThreads, 0, st>>>(fa(kShapeParticles));
  mark(c, SPH_KERNEL_BIN_SCATTER, 1);
  mark(c, SPH_KERNEL_BIN_RANK, 0);
  fused_rank_kernel<<<grid(kShapeRank), kThreads, 0, st>>>(fa(kShapeRank));
  mark(c, SPH_KERNEL_BIN_RANK, 1);
  mark(c, SPH_KERNEL_BIN_SCAN, 0);
  fused_items_count_kernel<<<grid(kShapeBuckets), kThreads, 0, st>>>(fa(kShapeBuckets));
  mark(c, SPH_KERNEL_BIN_SCAN, 1);
  scan(1);
  mark(c, SPH_KERNEL_BIN_SCAN, 0);
  fused_items_write_kernel<<<grid(kShapeCells), kThreads, 0, st>>>(fa(kShapeCells));
  mark(c, SPH_KERNEL_BIN_SCAN, 1);
  mark(c, SPH_KERNEL_BIN_GATHER, 0);
  if (fb.dim == 2)
    fused_gather_kernel<2><<<grid(kShapeParticles), kThreads, 0, st>>>(fa(kShapeParticles));
  else
    fused_gather_kernel<3><<<grid(kShapeParticles), kThreads, 0, st>>>(fa(kShapeParticles));
  mark(c, SPH_KERNEL_BIN_GATHER, 1);
  mark(c, SPH_KERNEL_BIN_SCAN, 0);
  fused_chunks_count_kernel<<<grid(kShapeBuckets), kThreads, 0, st>>>(fa(kShapeBuckets));
  mark(c, SPH_KERNEL_BIN_SCAN, 1);
  scan(2);
  return cudaGetLastError();
}

size_t scan_tmp_ints(int len) { return (size_t)((len + kScanTile - 1) / kScanTile) + 1; }

cudaError_t launch_scan(const LaunchCtx& c, const int* in, int* out, int len, int* tmp) {
  const int nblocks = (len + kScanTile - 1) / kScanTile;
  if (nblocks == 0) return cudaSuccess;
  mark(c, SPH_KERNEL_BIN_SCAN, 0);
  scan_reduce_kernel<<<nblocks, kScanThreads, 0, c.stream>>>(in, len, tmp);
  scan_blocks_kernel<<<1, 1024, 0, c.stream>>>(tmp, nblocks);
  scan_apply_kernel<<<nblocks, kScanThreads, 0, c.stream>>>(in, out, len, tmp);
  mark(c, SPH_KERNEL_BIN_SCAN, 1, 3);
  return cudaGetLastError();
}

cudaError_t launch_binning(const LaunchCtx& c, const State& cur, const State& alt,
                           const Geometry& g, const Consts& k, const BinScratch& b, int cap,
                           int step_mode, int gather_mode) {
  if (cap <= 0) return cudaSuccess;
  const int blocks = (cap + kThreads - 1) / kThreads;
  const int nbuckets = g.key_max + 3;
  cudaError_t e = cudaMemsetAsync(b.counts, 0, sizeof(int) * (size_t)nbuckets, c.stream);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(b.d_nrem, 0, sizeof(int), c.stream);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(b.cell_fluid, 0, sizeof(int) * (size_t)nbuckets, c.stream);
  if (e != cudaSuccess) return e;
  mark(c, SPH_KERNEL_BIN_KEYS, 0);
  if (k.dim == 2)
    bin_keys_kernel<2><<<blocks, kThreads, 0, c.stream>>>(cur, g, k, b, step_mode);
  else
    bin_keys_kernel<3><<<blocks, kThreads, 0, c.stream>>>(cur, g, k, b, step_mode);
  mark(c, SPH_KERNEL_BIN_KEYS, 1);
  mark(c, SPH_KERNEL_BIN_REMOVE, 0);
  bin_remove_kernel<<<1, 1024, 0, c.stream>>>(b);
  mark(c, SPH_KERNEL_BIN_REMOVE, 1);
  e = launch_scan(c, b.counts, b.cell_start, nbuckets, b.scan_tmp);
  if (e != cudaSuccess) return e;
  mark(c, SPH_KERNEL_BIN_SCATTER, 0);
  bin_scatter_kernel<<<blocks, kThreads, 0, c.stream>>>(cur, g, b);
  mark(c, SPH_KERNEL_BIN_SCATTER, 1);
  mark(c, SPH_KERNEL_BIN_RANK, 0);
  const int rank_blocks = (g.key_max + (kThreads / 32) - 1) / (kThreads / 32);
  bin_rank_kernel<<<rank_blocks, kThreads, 0, c.stream>>>(g, b);
  mark(c, SPH_KERNEL_BIN_RANK, 1);
  // work list of the pair passes (cells are final once the starts exist)
  mark(c, SPH_KERNEL_BIN_SCAN, 0);
  items_count_kernel<<<(nbuckets + kThreads - 1) / kThreads, kThreads, 0, c.stream>>>(g, b);
  mark(c, SPH_KERNEL_BIN_SCAN, 1);
  e = launch_scan(c, b.counts, b.item_off, nbuckets, b.scan_tmp);
  if (e != cudaSuccess) return e;
  mark(c, SPH_KERNEL_BIN_SCAN, 0);
  items_write_kernel<<<(g.key_max + kThreads - 1) / kThreads, kThreads, 0, c.stream>>>(g, b);
  mark(c, SPH_KERNEL_BIN_SCAN, 1);
  mark(c, SPH_KERNEL_BIN_GATHER, 0);
  if (k.dim == 2)
    bin_gather_kernel<2><<<blocks, kThreads, 0, c.stream>>>(cur, alt, g, k, b, gather_mode);
  else
    bin_gather_kernel<3><<<blocks, kThreads, 0, c.stream>>>(cur, alt, g, k, b, gather_mode);
  mark(c, SPH_KERNEL_BIN_GATHER, 1);
  if (b.ck_mask) {
    // after the gather: it counts each cell's fluid particles
    mark(c, SPH_KERNEL_BIN_SCAN, 0);
    chunks_count_kernel<<<(nbuckets + kThreads - 1) / kThreads, kThreads, 0, c.stream>>>(g, b);
    mark(c, SPH_KERNEL_BIN_SCAN, 1);
    e = launch_scan(c, b.counts, b.chunk_off, nbuckets, b.scan_tmp);
    if (e != cudaSuccess) return e;
  }
  return cudaGetLastError();
}

}  // namespace sphgpu
