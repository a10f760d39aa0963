// sph_tile64.cu -- the FP64 density and force passes of a step with every
// pair evaluated once.
//
// Each pair's contribution is a symmetric scalar times a vector that changes
// sign with the direction, exactly in IEEE arithmetic: the kernel distance r
// (squares of negated differences), m W(r), rho_p + rho_q and
// P_p/rho_p^2 + P_q/rho_q^2 (commutative additions), (v_p - v_q).(x_p - x_q)
// (products of two negated differences), hence the viscosity term, the
// pressure factor cf and the XSPH factor wx.  Both directions of a pair
// therefore contribute bit-identical factors, and a target's sums only need
// them in its own neighbour order.  The pair set is symmetric too: outside
// the FP32 band the FP32 decision equals the exact test, inside the band it
// is the exact test, which squares the differences.
//
// Rows (CSR, sized from the counts): every target's row holds its
// neighbours (neighbour index, distance, two factors; a wall's row its fluid
// neighbours).  The neighbours in the reference's order (core.jl:96-105) are
// the slots of key_diff in turn, each slot's cell in stored order, so the row
// is one segment per slot: the segment of (target i, slot c) holds i's hits
// in cell key(i) + key_diff[c], in ascending index order.
//
// Tiles: one warp per (cell a, forward slot c >= the centre slot), with
// b = a + key_diff[c].  The tile owns the segments (p in a, slot c) and
// (q in b, slot mirror(c)), where mirror(c) = n_diff - 1 - c is the slot from
// b back to a; every segment has exactly one writer, so nothing is atomic
// but the pair list's tail.  A tile classifies a x b in blocks of 32 x 32:
// lane u tests column q_u against the 32 staged rows with packed FP32x2
// arithmetic (bit i of its column mask); the row masks are the transposes (a
// butterfly bit transpose).  The rank of q in p's segment is the number of
// p's hits in the earlier column blocks (a cursor) plus the bits of p's row
// mask below q, and likewise for p in q's segment.  The tile of the cell
// itself (c = centre) takes each unordered pair once (p < q); its diagonal
// blocks are symmetric.
//
// Passes of a step (launch order):
//   tiles    classify once: rseg := hits per (target, slot); the pair list
//            (p, q, both ranks, slot, wall bits)
//   count    hit_count (the row length), c4 = the row in 128-byte units,
//            rseg := each segment's first entry relative to the row's start;
//            the fixed-point positions (xfix and the records' first halves);
//            the walls' lists for the wall pressure
//   scan     row_base := exclusive prefix of c4 over the particles
//   offsets  rseg += the row's start 4 row_base; rows beyond row_cap send
//            every target to the traversal (and tell the host)
//   density  per pair: m W, r and t into both rows (at rseg + rank); a
//            wall's entry gets W and g.(x_w - x_f) instead
//   [sum]    sph_pair64.cu: rho = the row's sum, self term, EOS
//   [wall]   sph_pair64.cu: each wall's pressure over its row (fluid
//            neighbours, the kernel value from the stored t)
//   records  every particle's FxRec from the current fields
//   force    per pair: cf and wx into both rows (a fluid-wall pair only into
//            the fluid target's row: walls are not force targets)
//   [sum]    sph_pair64.cu: a += cf d, xs += -wx dv over the row
//
// A row with a segment of more than kSegMax hits (the 10-bit ranks), or a
// target next to a cell of more than 65535 particles (the tiles' 16-bit local
// indices), is marked overflowed by the count; its sum passes traverse
// instead.  A pair list longer than pair_cap, or rows beyond row_cap, send
// every target to the traversal.
//
// The pair kernels form position differences, the kernel distance's square
// root and the force's reciprocals on the integer pipes, correctly rounded
// (sph_common.cuh: fx_diff, isqrt_rn, ircp_rn).  Built with --fmad=false like
// sph_pair64.cu: the FP64 expressions below round where they are written, in
// the oracle's order.
#include <algorithm>

#include "sph_cellwarp.cuh"
#include "sph_launch.h"
#include "sphgpu.h"

namespace sphgpu {

namespace {

constexpr int kTileWarps = 4;
constexpr int kTileList = 512;         // pairs buffered per warp before they are listed
constexpr float kTileFar = 1.0e18f;    // coordinate of an empty staging slot
// pair_m: rank in p's segment (10 bits), rank in q's segment (10), slot (5),
// p is a wall, q is a wall.  A rank of kRankNone (> kSegMax) marks a side
// beyond what a rank addresses (that target's row is not used).  Wall rows
// hold their fluid neighbours (pairs of two walls are not listed) for the
// wall pressure.
constexpr unsigned kRankNone = 1023u;
static_assert(kSegMax < (int)kRankNone, "ranks up to kSegMax must be encodable");
constexpr unsigned kPWall = 1u << 25, kQWall = 1u << 26;

struct TileShared {
  // rows: cell-relative positions minus b's offset (pairs of rows are read
  // as one 64-bit word by the packed classification)
  float rx[32], ry[32], rz[32];
  unsigned rmask[32];     // row masks of the current block (bit u = column u)
  int rcur[32];           // row cursors at the start of the current block
  uint2 list[kTileList];  // pairs: (p_local | q_local << 16, pair_m)
};

// 32 x 32 bit transpose across the warp: lane u holds column u's mask (bit i
// = row i) on entry and row u's mask (bit i = column i) on return.  Each
// stage swaps the off-diagonal blocks of width j.
__device__ __forceinline__ unsigned warp_transpose(unsigned x, int lane) {
  const unsigned m[5] = {0x0000ffffu, 0x00ff00ffu, 0x0f0f0f0fu, 0x33333333u, 0x55555555u};
#pragma unroll
  for (int st = 0; st < 5; ++st) {
    const int j = 16 >> st;
    const unsigned y = __shfl_xor_sync(0xffffffffu, x, j);
    x = (lane & j) ? ((x & ~m[st]) | ((y >> j) & m[st])) : ((x & m[st]) | ((y << j) & ~m[st]));
  }
  return x;
}

// Appends the warp's buffered pairs to the pair list.
__device__ __forceinline__ void tile_emit(const BinScratch& b, const TileShared& sh, int lane,
                                          int n, int sa, int sb) {
  unsigned long long base = 0;
  if (lane == 0) base = atomicAdd(b.d_npairs, (unsigned long long)n);
  base = __shfl_sync(0xffffffffu, base, 0);
  if (base + (unsigned long long)n > (unsigned long long)b.pair_cap) {
    if (lane == 0) *b.d_pover = 1;
    return;
  }
  for (int e = lane; e < n; e += 32) {
    const uint2 en = sh.list[e];
    const size_t o = (size_t)base + e;
    b.pair_p[o] = sa + (int)(en.x & 0xffffu);
    b.pair_q[o] = sb + (int)(en.x >> 16);
    b.pair_m[o] = en.y;
  }
}

// One tile: cell a = [sa, sa + na), slot c, cell nk = [sb, sb + nb).
template <int DIM>
__device__ __forceinline__ void tile_run(const State& s, const Geometry& g, const Consts& k,
                                         const BinScratch& b, TileShared& sh, int lane, int a,
                                         int nk, int c, int sa, int na, int sb, int nb) {
  const unsigned full = 0xffffffffu;
  const int nd = g.n_diff;
  const bool self = c == (nd >> 1);
  const int mc = nd - 1 - c;
  const int cap = kSegMax + 1;  // ranks below this are addressable
  const unsigned below = lanemask_lt();
  // b's origin relative to a's (the traversal's cw_offset)
  int acx, acy, acz, bcx, bcy, bcz;
  decode_key(g, a, acx, acy, acz);
  decode_key(g, nk, bcx, bcy, bcz);
  const float ox = (float)(bcx - acx) * k.cellf;
  const float oy = (float)(bcy - acy) * k.cellf;
  const float oz = (float)(bcz - acz) * k.cellf;
  const int nA = (na + 31) >> 5, nB = (nb + 31) >> 5;
  int ln = 0;  // pairs buffered
  for (int ia = 0; ia < nA; ++ia) {
    const int ma = min(32, na - 32 * ia);
    const int p = sa + 32 * ia + lane;
    float4 pr = make_float4(kTileFar, kTileFar, kTileFar, __int_as_float(-1));
    int rc = 0;  // this lane's row cursor: p's hits in the blocks so far
    if (lane < ma) {
      pr = __ldg(&s.pl[p]);
      // the row's position relative to b's origin, rounded as the
      // traversal's (xl_p - offset)
      pr.x = pr.x - ox;
      pr.y = pr.y - oy;
      pr.z = pr.z - oz;
      // in the own cell's tile, earlier blocks counted p's hits as a column
      if (self && ia > 0) rc = (int)b.rseg[rseg_at(b, p, c)];
    }
    __syncwarp();
    sh.rx[lane] = pr.x;
    sh.ry[lane] = pr.y;
    sh.rz[lane] = pr.z;
    const unsigned afl = __ballot_sync(full, lane < ma && __float_as_int(pr.w) == kFluid);
    __syncwarp();
    for (int jb = self ? ia : 0; jb < nB; ++jb) {
      const bool diag = self && jb == ia;
      const int mb = min(32, nb - 32 * jb);
      const int q = sb + 32 * jb + lane;
      // this lane's column particle (the diagonal block: the row itself,
      // offset 0)
      float4 pc = pr;
      if (!diag)
        pc = lane < mb ? __ldg(&s.pl[q])
                       : make_float4(kTileFar, kTileFar, kTileFar, __int_as_float(-1));
      const bool qfl = lane < mb && __float_as_int(pc.w) == kFluid;
      unsigned cm = 0u, bm = 0u;
      if (lane < mb) {
        // two rows per packed operation; empty row slots are far away.  Any
        // FP32 rounding of the squared distance is within the band's margin.
        // The decisions are the signs of s_hi - ss (set: beyond the support)
        // and ss - s_lo (set: below the band), exact in FP32, funnel-shifted
        // into the masks from row 31 down to row 0.
        const unsigned long long cx = f2_pack(pc.x, pc.x), cy = f2_pack(pc.y, pc.y);
        const unsigned long long cz = f2_pack(pc.z, pc.z);
        const unsigned long long shi = f2_pack(k.s_hi, k.s_hi), slo = f2_pack(k.s_lo, k.s_lo);
        const unsigned long long* rx2 = reinterpret_cast<const unsigned long long*>(sh.rx);
        const unsigned long long* ry2 = reinterpret_cast<const unsigned long long*>(sh.ry);
        const unsigned long long* rz2 = reinterpret_cast<const unsigned long long*>(sh.rz);
        unsigned out = 0u, low = 0u;
#pragma unroll
        for (int i2 = 15; i2 >= 0; --i2) {
          const unsigned long long dx = f2_sub(rx2[i2], cx);
          const unsigned long long dy = f2_sub(ry2[i2], cy);
          unsigned long long ss = f2_fma(dy, dy, f2_mul(dx, dx));
          if (DIM == 3) {
            const unsigned long long dz = f2_sub(rz2[i2], cz);
            ss = f2_fma(dz, dz, ss);
          }
          const unsigned long long dh = f2_sub(shi, ss);
          const unsigned long long dl = f2_sub(ss, slo);
          out = __funnelshift_l((unsigned)(dh >> 32), out, 1);
          out = __funnelshift_l((unsigned)dh, out, 1);
          low = __funnelshift_l((unsigned)(dl >> 32), low, 1);
          low = __funnelshift_l((unsigned)dl, low, 1);
        }
        cm = ~out;
        bm = ~low & cm;
        // a particle is not its own neighbour (core.jl:105)
        const int di = q - (sa + 32 * ia);
        if (di >= 0 && di < 32) {
          cm &= ~(1u << di);
          bm &= ~(1u << di);
        }
        // a pair of walls takes part in neither pass
        if (!qfl) {
          cm &= afl;
          bm &= afl;
        }
      }
      // band candidates: the reference's FP64 test, all lanes together
      while (__any_sync(full, bm != 0u)) {
        if (bm) {
          const int i = __ffs(bm) - 1;
          bm &= bm - 1u;
          const int pi = sa + 32 * ia + i;
          double xr[3];
          xr[0] = __ldg(&s.x[0][pi]);
          xr[1] = __ldg(&s.x[1][pi]);
          xr[2] = DIM == 3 ? __ldg(&s.x[2][pi]) : 0.0;
          if (!within_rn<DIM>(s, k, xr, q)) cm &= ~(1u << i);
        }
      }
      // row masks (bit u = column u); the diagonal block is symmetric
      const unsigned rm = diag ? cm : warp_transpose(cm, lane);
      // the column's cursor (in the diagonal block: the particle's own)
      int cc = rc;
      size_t cj = 0;
      if (!diag && lane < mb) {
        cj = rseg_at(b, q, mc);
        cc = ia == 0 ? 0 : (int)b.rseg[cj];
      }
      sh.rmask[lane] = rm;
      sh.rcur[lane] = rc;
      __syncwarp();
      // the block's pairs with their ranks in both segments.  A column takes
      // its rows in ascending order, so its rank in the column's segment
      // counts up from the cursor (in the diagonal block the bits below the
      // lane are all of the column's bits below each row taken).  A side
      // without a row entry (a wall, or a rank beyond kSegMax) is marked
      // kRankNone; the pair kernels skip a pair with neither.
      unsigned em = diag ? (cm & below) : cm;
      const unsigned lbase = (unsigned)(32 * ia) | ((unsigned)(32 * jb + lane) << 16);
      const unsigned mbase = ((unsigned)c << 20) | (qfl ? 0u : kQWall);
      const int cnt = __popc(em);
      int incl = cnt;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(full, incl, o);
        if (lane >= o) incl += t;
      }
      const int total = __shfl_sync(full, incl, 31);
      if (ln + total > kTileList) {
        __syncwarp();
        tile_emit(b, sh, lane, ln, sa, sb);
        ln = 0;
        __syncwarp();
      }
      if (total <= kTileList) {
        // each lane writes its column's pairs into its own slice of the list
        int slot = ln + incl - cnt;
        int qrank = cc;
        while (em) {
          const int i = __ffs(em) - 1;
          em &= em - 1u;
          const bool pfl = (afl >> i) & 1u;
          const int v = sh.rcur[i] + __popc(sh.rmask[i] & below);
          const unsigned pr_ = v < cap ? (unsigned)v : kRankNone;
          const unsigned qr_ = qrank < cap ? (unsigned)qrank : kRankNone;
          ++qrank;
          sh.list[slot++] = make_uint2(lbase + (unsigned)i,
                                       pr_ | (qr_ << 10) | mbase | (pfl ? 0u : kPWall));
        }
        ln += total;
      } else {
        // more pairs than the buffer holds (dense clusters): whole warps of
        // pairs at a time, emitted as the buffer fills
        int qrank = cc;
        for (;;) {
          const bool has = em != 0u;
          if (__ballot_sync(full, has) == 0u) break;
          unsigned meta = 0u, loc = 0u;
          if (has) {
            const int i = __ffs(em) - 1;
            em &= em - 1u;
            const bool pfl = (afl >> i) & 1u;
            const int v = sh.rcur[i] + __popc(sh.rmask[i] & below);
            const unsigned pr_ = v < cap ? (unsigned)v : kRankNone;
            const unsigned qr_ = qrank < cap ? (unsigned)qrank : kRankNone;
            ++qrank;
            meta = pr_ | (qr_ << 10) | mbase | (pfl ? 0u : kPWall);
            loc = lbase + (unsigned)i;
          }
          const unsigned hb = __ballot_sync(full, has);
          if (ln + __popc(hb) > kTileList) {
            __syncwarp();
            tile_emit(b, sh, lane, ln, sa, sb);
            ln = 0;
            __syncwarp();
          }
          if (has) sh.list[ln + __popc(hb & below)] = make_uint2(loc, meta);
          ln += __popc(hb);
        }
      }
      if (!diag && lane < mb) b.rseg[cj] = (unsigned)(cc + __popc(cm));
      __syncwarp();
      rc += __popc(rm);
    }
    if (lane < ma) b.rseg[rseg_at(b, p, c)] = (unsigned)rc;
  }
  if (ln > 0) {
    __syncwarp();
    tile_emit(b, sh, lane, ln, sa, sb);
  }
  __syncwarp();
}

// Warps stride over the tile slots (work item, forward slot); a tile is
// taken by its cell's first item.
template <int DIM>
__global__ void __launch_bounds__(32 * kTileWarps, 10) tile_kernel(State s, Geometry g, Consts k,
                                                               BinScratch b, int warps_total) {
  __shared__ TileShared shared[kTileWarps];
  TileShared& sh = shared[threadIdx.x >> 5];
  const int lane = threadIdx.x & 31;
  const int ctr = g.n_diff >> 1;
  const int nf = ctr + 1;
  const long long n_slots = (long long)__ldg(&b.item_off[g.key_max + 1]) * nf;
  for (long long w = (long long)blockIdx.x * kTileWarps + (threadIdx.x >> 5); w < n_slots;
       w += warps_total) {
    const int item = (int)(w / nf);
    const int c = ctr + (int)(w - (long long)item * nf);
    const int first = __ldg(&b.items[item]).x;
    const int a = __ldg(&s.cell[first]);
    const int sa = __ldg(&b.cell_start[a]);
    if (first != sa) continue;
    const int nk = a + g.key_diff[c];
    if (nk < 1 || nk > g.key_max) continue;  // core.jl:98
    if (__ldg(&b.cell_fluid[a]) == 0 && __ldg(&b.cell_fluid[nk]) == 0) continue;
    const int na = __ldg(&b.cell_start[a + 1]) - sa;
    const int sb = __ldg(&b.cell_start[nk]);
    const int nb = __ldg(&b.cell_start[nk + 1]) - sb;
    if (nb == 0 || na > 0xffff || nb > 0xffff) continue;
    tile_run<DIM>(s, g, k, b, sh, lane, a, nk, c, sa, na, sb, nb);
  }
}

// Particle i's part of row_count_kernel: returns its row in units of four
// entries and, for a wall, its list (1: with fluid neighbours, 2: without, 0:
// its row is not used).
__device__ __forceinline__ int row_count_body(const State& s, const Geometry& g, const Consts& k,
                                              const BinScratch& b, int i, int& wall) {
  long long X[3] = {0, 0, 0};
  for (int d = 0; d < k.dim; ++d) {
    X[d] = fx_fix(s.x[d][i], k.fx_k);
    b.xfix[d][i] = X[d];
  }
  // the position half of the particle's record, for the density pair kernel
  asm volatile("st.global.v4.b64 [%0], {%1, %2, %3, %4};" ::"l"(b.frec + i), "l"(X[0]),
               "l"(X[1]), "l"(X[2]), "d"(s.v[0][i])
               : "memory");
  const int key = s.cell[i];
  const int nd = g.n_diff;
  bool over = __ldg(&b.cell_start[key + 1]) - __ldg(&b.cell_start[key]) > 0xffff;
  const bool own_fluid = __ldg(&b.cell_fluid[key]) != 0;
  unsigned* seg = b.rseg + i;  // seg[c * rseg_stride]: slot-major
  // every slot's count first (independent loads), then the relative offsets
  int cnt[27];
#pragma unroll
  for (int c = 0; c < 27; ++c) {
    cnt[c] = 0;
    if (c < nd) {
      const int nk = key + g.key_diff[c];
      if (nk >= 1 && nk <= g.key_max) {
        const int m = __ldg(&b.cell_start[nk + 1]) - __ldg(&b.cell_start[nk]);
        if (m > 0xffff) over = true;
        // a tile between two cells without fluid is skipped (no pair of it
        // involves a fluid particle), so its counts are not written
        else if (m > 0 && (own_fluid || __ldg(&b.cell_fluid[nk]) != 0))
          cnt[c] = (int)seg[(size_t)c * b.rseg_stride];
      }
    }
  }
  int run = 0;
#pragma unroll
  for (int c = 0; c < 27; ++c) {
    if (c < nd) {
      if (cnt[c] > kSegMax) over = true;
      // the segment's first entry relative to the row's start (the offsets
      // pass adds the start, 4 row_base[i], once the scan has it)
      seg[(size_t)c * b.rseg_stride] = (unsigned)run;
      run += cnt[c];
    }
  }
  const bool is_wall = s.type[i] == kWall;
  if (over) {
    // an overflowed target has no row: the pair passes treat its side like
    // one beyond the rows and its sums traverse
    for (int c = 0; c < nd; ++c) seg[(size_t)c * b.rseg_stride] = kNoRow;
    b.hit_count[i] = kRowOver;
    *b.d_rover = 1;
    wall = 0;
    return 0;
  }
  b.hit_count[i] = run;
  wall = is_wall ? (run > 0 ? 1 : 2) : 0;
  return (run + 3) >> 2;
}

// Each particle's row length from its per-slot counts (a wall's row holds
// its fluid neighbours), the row in 128-byte units for the scan, and the
// positions' fixed-point copies for the pair kernels.  Threads up to `cap`
// (inclusive) write c4, so that the scan's last element gives the total.
__global__ void __launch_bounds__(256) row_count_kernel(State s, Geometry g, Consts k,
                                                        BinScratch b, int cap) {
  __shared__ int block_sum;
  if (threadIdx.x == 0) block_sum = 0;
  __syncthreads();
  const int n = *b.d_n;
  const int i = blockIdx.x * 256 + threadIdx.x;
  int wall = 0;
  const int c4 = i < n ? row_count_body(s, g, k, b, i, wall) : 0;
  if (i <= cap) b.c4[i] = c4;
  // the wall pressure's lists (one atomic per warp and list; the order
  // within a list does not matter: every wall's sum is its own)
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  for (int l = 1; l <= 2; ++l) {
    const unsigned m = __ballot_sync(full, wall == l);
    if (!m) continue;
    const int leader = __ffs(m) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(&b.d_nwall[l - 1], __popc(m));
    base = __shfl_sync(full, base, leader);
    if (wall == l) {
      const int j = base + __popc(m & lanemask_lt());
      b.wall_list[l == 1 ? j : b.wall_cap - 1 - j] = i;
    }
  }
  // the exact total (64-bit) beside the scan's int32 one
  const int ws = __reduce_add_sync(0xffffffffu, c4);
  if ((threadIdx.x & 31) == 0 && ws) atomicAdd(&block_sum, ws);
  __syncthreads();
  if (threadIdx.x == 0 && block_sum) atomicAdd(b.d_rowsum, (unsigned long long)block_sum);
}

// Each segment's absolute first entry: the row's start (4 row_base[i], the
// scan of c4) added to the relative offsets the row count wrote, all 27
// loaded before any is stored.  Rows beyond row_cap: every target traverses
// this pass (the pair list's overflow flag) and the host, which reads
// need_host between passes, grows the rows.  The fit is decided on the exact
// 64-bit total; when it fits (row_cap < 2^32 entries), the int32 scan cannot
// have wrapped.
__global__ void __launch_bounds__(256) row_offsets_kernel(Geometry g, BinScratch b) {
  const int n = *b.d_n;
  const int i = blockIdx.x * 256 + threadIdx.x;
  if (i >= n) return;
  const unsigned long long total = 4ull * *b.d_rowsum;
  if (total > (unsigned long long)b.row_cap) {
    if (i == 0) {
      *b.d_pover = 1;
      if (b.need_host && *b.need_host < total) *b.need_host = total;
    }
    return;
  }
  const int nd = g.n_diff;
  unsigned* seg = b.rseg + i;
  unsigned rel[27];
#pragma unroll
  for (int c = 0; c < 27; ++c) rel[c] = c < nd ? seg[(size_t)c * b.rseg_stride] : 0u;
  const unsigned base = 4u * __ldg(&b.row_base[i]);  // < row_cap < 2^32
#pragma unroll
  for (int c = 0; c < 27; ++c)
    if (c < nd && rel[c] != kNoRow) seg[(size_t)c * b.rseg_stride] = base + rel[c];
}

// The force records (FxRec) of every particle from the SoA state: the
// density pass's fixed-point copies, the velocities after the step's first
// kick, the densities and P/rho^2 after the EOS and the wall pressure.
template <int DIM>
__global__ void __launch_bounds__(256) frec_build_kernel(State s, BinScratch b) {
  const int n = *b.d_n;
  const int i = blockIdx.x * 256 + threadIdx.x;
  if (i >= n) return;
  const long long X0 = b.xfix[0][i], X1 = b.xfix[1][i];
  const long long X2 = DIM == 3 ? b.xfix[2][i] : 0;
  const double v0 = s.v[0][i], v1 = s.v[1][i];
  const double v2 = DIM == 3 ? s.v[2][i] : 0.0;
  FxRec* r = b.frec + i;
  asm volatile("st.global.v4.b64 [%0], {%1, %2, %3, %4};" ::"l"(r), "l"(X0), "l"(X1), "l"(X2),
               "d"(v0)
               : "memory");
  asm volatile("st.global.v4.b64 [%0], {%1, %2, %3, %4};" ::"l"(&r->v1), "d"(v1), "d"(v2),
               "d"(s.rho[i]), "d"(s.Pr[i])
               : "memory");
}

// The FP64 evaluation of the listed pairs into the rows (PH 0: density,
// 1: force).  Threads stride over the list.  A side writes its entry only
// when its target has a row (overflowed targets have none) and, in the force
// pass, is fluid; every entry is written whole.
template <int DIM, int PH>
__global__ void __launch_bounds__(256, PH == 0 ? 6 : 5) pair_list_kernel(State s, Geometry g, Consts k,
                                                        BinScratch b, int threads_total) {
  if (*b.d_pover) return;  // every target traverses
  const long long np = (long long)*b.d_npairs;
  const int nd = g.n_diff;
  int av = 0;
  for (long long e = (long long)blockIdx.x * 256 + threadIdx.x; e < np; e += threads_total) {
    const int p = __ldg(&b.pair_p[e]);
    const int q = __ldg(&b.pair_q[e]);
    const unsigned m = __ldg(&b.pair_m[e]);
    const int c = (int)((m >> 20) & 31u);
    const bool fp = (m & kPWall) == 0u, fq = (m & kQWall) == 0u;
    // entry positions: the segment's first entry plus the rank (a rank of
    // kRankNone, or a target without a row, writes nothing); the density
    // pass fills wall rows too (the wall pressure's neighbours), the force
    // pass fluid rows only
    const unsigned rp = m & 1023u, rq = (m >> 10) & 1023u;
    unsigned bp = kNoRow, bq = kNoRow;
    if ((PH == 0 || fp) && rp != kRankNone) bp = __ldg(&b.rseg[rseg_at(b, p, c)]);
    if ((PH == 0 || fq) && rq != kRankNone) bq = __ldg(&b.rseg[rseg_at(b, q, nd - 1 - c)]);
    const bool wp = bp != kNoRow, wq = bq != kNoRow;
    if (!wp && !wq) continue;
    RowEntry* const ep = b.rows + (wp ? (size_t)bp + rp : 0);
    RowEntry* const eq = b.rows + (wq ? (size_t)bq + rq : 0);
    const unsigned long long qbits = (unsigned)q | (fq ? 0u : 0x80000000u);
    const unsigned long long pbits = (unsigned)p | (fp ? 0u : 0x80000000u);
    if (PH == 0) {
      // kdist64's distance, the separations formed exactly on the integer pipes
      long long PX0, PX1, PX2, QX0, QX1, QX2;
      double pv0, qv0;
      frec_load_x(b.frec + p, PX0, PX1, PX2, pv0);
      frec_load_x(b.frec + q, QX0, QX1, QX2, qv0);
      const double d0 = fx_sep2(PX0, &s.x[0][p], QX0, &s.x[0][q], k.fx_k);
      const double d1 = fx_sep2(PX1, &s.x[1][p], QX1, &s.x[1][q], k.fx_k);
      double ss = __fma_rn(d1, d1, d0 * d0);
      double d2 = 0.0;
      if (DIM == 3) {
        d2 = fx_sep2(PX2, &s.x[2][p], QX2, &s.x[2][q], k.fx_k);
        ss = __fma_rn(d2, d2, ss);
      }
      const double r = isqrt_rn(ss);
      const double t = ker_t(k, r);
      const double t2 = t * t;
      const double w = (t2 * t2) * __fma_rn(k.mcw4, t, k.mcw5);  // m W
      if (fp && fq) {
        // t = 1 - r/H rides in the entry's spare slot, so that the force
        // pass of this binning starts its kernel derivative from it
        if (wp) row_store(ep, qbits, w, r, t);
        if (wq) row_store(eq, pbits, w, r, t);
      } else {
        // a fluid-wall pair: the fluid target's entry as above; the wall's
        // entry holds what its pressure sums (Proc64::rows): the kernel
        // value without the mass and g.(x_w - x_f).  gd below is
        // g.(x_p - x_q); the wall's is it when p is the wall and its
        // negation (exact) when q is
        const double wc = (k.cw * (t2 * t2)) * __fma_rn(-4.0, t, 5.0);
        double gd = __fma_rn(k.g[1], d1, k.g[0] * d0);
        if (DIM == 3) gd = __fma_rn(k.g[2], d2, gd);
        if (wp) row_store(ep, qbits, fp ? w : wc, fp ? r : gd, t);
        if (wq) row_store(eq, pbits, fq ? w : wc, fq ? r : -gd, t);
      }
    } else {
      // m W, r and t as the density pass of this binning stored them
      const RowEntry en = row_load(wp ? ep : eq);
      const double w = en.a, r = en.b, t = en.c;
      const double t2 = t * t;
      const double ker = k.mcr * (t2 * t);  // m rDW
      if (fp && fq) {
        // pressure (collapse_symplectic.jl:114-118) + Monaghan viscosity +
        // XSPH, in p's direction (q's is the same factor); both particles'
        // force records (frec_build_kernel), the (v1, v2, rho, P/rho^2)
        // halves first
        double sp, rs, dv1, dv2;
        {
          double pv1, pv2, prho, ppr, qv1, qv2, qrho, qpr;
          frec_load_v(b.frec + p, pv1, pv2, prho, ppr);
          frec_load_v(b.frec + q, qv1, qv2, qrho, qpr);
          sp = ppr + qpr;
          rs = prho + qrho;
          dv1 = pv1 - qv1;
          dv2 = DIM == 3 ? pv2 - qv2 : 0.0;
        }
        long long PX0, PX1, PX2, QX0, QX1, QX2;
        double pv0, qv0;
        frec_load_x(b.frec + p, PX0, PX1, PX2, pv0);
        frec_load_x(b.frec + q, QX0, QX1, QX2, qv0);
        const double d0 = fx_sep2(PX0, &s.x[0][p], QX0, &s.x[0][q], k.fx_k);
        const double d1 = fx_sep2(PX1, &s.x[1][p], QX1, &s.x[1][q], k.fx_k);
        const double dv0 = pv0 - qv0;
        double vdx = __fma_rn(dv1, d1, dv0 * d0);
        if (DIM == 3) {
          const double d2 = fx_sep2(PX2, &s.x[2][p], QX2, &s.x[2][q], k.fx_k);
          vdx = __fma_rn(dv2, d2, vdx);
        }
        const double inv_rb = two_over(rs);
        double pi = 0.0;
        if (lt0(vdx)) {
          // mu = h v.x / (r^2 + eta^2), r^2 + eta^2 as one fused multiply-add,
          // the quotient as a product with the reciprocal
          pi = ((k.ca * vdx) * ircp_rn(__fma_rn(r, r, k.eta2))) * inv_rb;
          // one count per direction whose row is summed
          av += (wp ? 1 : 0) + (wq ? 1 : 0);
        }
        const double cf = -ker * (sp + pi);
        const double wx = w * inv_rb;  // m W / rho_bar
        if (wp) row_store(ep, qbits, cf, wx);
        if (wq) row_store(eq, pbits, cf, wx);
      } else {
        // fluid-wall: the pressure term with the wall pressure, into the
        // fluid target's row (a wall has no row entry)
        const double sp = __ldg(&s.Pr[p]) + __ldg(&s.Pr[q]);
        const double cf = -ker * sp;
        if (wp) row_store(ep, qbits, cf, 0.0);
        if (wq) row_store(eq, pbits, cf, 0.0);
      }
    }
  }
  if (PH == 1) cw_warp_add(b.d_cat + kCatForceAV, av);
}

template <int DIM>
cudaError_t tiles_dim(const LaunchCtx& c, const State& s, const Geometry& g, const Consts& k,
                      const BinScratch& b, int cap, int phase) {
  const cudaStream_t st = c.stream;
  static const int tile_wave = resident_blocks(tile_kernel<DIM>, 32 * kTileWarps);
  static const int dens_wave = resident_blocks(pair_list_kernel<DIM, 0>, 256);
  static const int force_wave = resident_blocks(pair_list_kernel<DIM, 1>, 256);
  if (phase == 0) {
    const long long slots = (long long)b.max_items * (g.n_diff / 2 + 1);
    const int tb = (int)std::max(
        1LL, std::min<long long>((slots + kTileWarps - 1) / kTileWarps, tile_wave));
    // pair count, overflow flags, the rows' 64-bit total, the wall counts
    cudaMemsetAsync(b.d_npairs, 0, 32, st);
    tile_kernel<DIM><<<tb, 32 * kTileWarps, 0, st>>>(s, g, k, b, tb * kTileWarps);
    row_count_kernel<<<cap / 256 + 1, 256, 0, st>>>(s, g, k, b, cap);
    // the rows' starts: c4[0 .. cap] -> row_base (row_base[n] = the total);
    // the scan's launches are counted by the caller with the tile kernels
    const LaunchCtx quiet{st, nullptr, nullptr};
    const cudaError_t e = launch_scan(quiet, b.c4, (int*)b.row_base, cap + 1, b.pscan_tmp);
    if (e != cudaSuccess) return e;
    row_offsets_kernel<<<(cap + 255) / 256, 256, 0, st>>>(g, b);
    pair_list_kernel<DIM, 0><<<dens_wave, 256, 0, st>>>(s, g, k, b, dens_wave * 256);
  } else {
    frec_build_kernel<DIM><<<(cap + 255) / 256, 256, 0, st>>>(s, b);
    pair_list_kernel<DIM, 1><<<force_wave, 256, 0, st>>>(s, g, k, b, force_wave * 256);
  }
  return cudaGetLastError();
}

// sph_arith_check's kernel: one value per thread
__global__ void arith_check_kernel(int op, int k, int n, const double* a, const double* b,
                                   double* out) {
  const int i = blockIdx.x * 256 + threadIdx.x;
  if (i >= n) return;
  const double x = a[i];
  double r;
  if (op == 0) {
    const long long X = fx_fix(x, k), Y = fx_fix(b[i], k);
    r = (X == kFxNone || Y == kFxNone) ? fx_fallback(x, &b[i]) : fx_diff(X, Y, k);
  } else if (op == 1) {
    r = isqrt_rn(x);
  } else if (op == 2) {
    r = ircp_rn(x);
  } else {
    r = two_over(x);
  }
  out[i] = r;
}

}  // namespace

cudaError_t launch_tiles_fp64(const LaunchCtx& c, const State& s, const Geometry& g,
                              const Consts& k, const BinScratch& b, int cap, int phase) {
  if (cap <= 0) return cudaSuccess;
  return k.dim == 2 ? tiles_dim<2>(c, s, g, k, b, cap, phase)
                    : tiles_dim<3>(c, s, g, k, b, cap, phase);
}

}  // namespace sphgpu

extern "C" int sph_arith_check(int device, int op, int k, int n, const double* a, const double* b,
                               double* out) {
  if (n < 0 || op < 0 || op > 3) return SPH_ERR_ARG;
  if (n == 0) return SPH_OK;
  if (!a || !out || (op == 0 && !b)) return SPH_ERR_ARG;
  int prev = 0;
  if (cudaGetDevice(&prev) != cudaSuccess || cudaSetDevice(device) != cudaSuccess) {
    cudaGetLastError();
    return SPH_ERR_CUDA;
  }
  const size_t bytes = sizeof(double) * (size_t)n;
  double* d = nullptr;
  int rc = SPH_OK;
  if (cudaMalloc(&d, 3 * bytes) != cudaSuccess) {
    rc = SPH_ERR_NOMEM;
  } else if (cudaMemcpy(d, a, bytes, cudaMemcpyHostToDevice) != cudaSuccess ||
             (op == 0 && cudaMemcpy(d + n, b, bytes, cudaMemcpyHostToDevice) != cudaSuccess)) {
    rc = SPH_ERR_CUDA;
  } else {
    sphgpu::arith_check_kernel<<<(n + 255) / 256, 256>>>(op, k, n, d, d + n, d + 2 * (size_t)n);
    if (cudaGetLastError() != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess ||
        cudaMemcpy(out, d + 2 * (size_t)n, bytes, cudaMemcpyDeviceToHost) != cudaSuccess)
      rc = SPH_ERR_CUDA;
  }
  if (d) cudaFree(d);
  cudaGetLastError();
  cudaSetDevice(prev);
  return rc;
}
