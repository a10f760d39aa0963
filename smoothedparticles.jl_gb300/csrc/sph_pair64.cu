// sph_pair64.cu -- the FP64 pair passes: _apply_binary! (core.jl:94-112) for
// the built-in operators, sum(sys, func, x / p) (core.jl:240-291) and the
// neighbour-pair listing used by the parity tests.
//
// Built with --fmad=false: every FP64 expression rounds exactly where it is
// written, in the order the CPU restatement uses, so results are bit-identical
// to it (IEEE division and square root are correctly rounded on both sides).
//
// The density and force passes of a step evaluate each pair once
// (sph_tile64.cu) and sum every target's row here, in the reference's
// order; targets whose rows overflowed, and the other operators, use the
// per-target traversal of sph_cellwarp.cuh (cell-aligned warps,
// shared-memory staged candidates, FP32 classification with an FP64 band
// test, per-target hit lists processed in order by every lane together).
// The FP64 pipe is the bound of these passes (1/58 of the FP32 rate on
// GB300), so the evaluation order below keeps FP64 operations per hit few:
// mass folded into the kernel constants, fused multiply-adds for the force
// sums, integer tests of x > 1 and v.x < 0, 2/(rho_p + rho_q) from a
// correctly rounded reciprocal.  The CPU restatement evaluates the same
// expressions.
//
// Why the FP32 classification is exact: positions are stored relative to
// their cell's origin, |xl| < 1.02 h; the neighbour-cell offset is an integer
// multiple of fl32(h).  The separation is formed as (xl_p - offset) - xl_q,
// three roundings of magnitudes below 2.1 h, so each component differs from
// the true separation by at most 8 * 2^-24 h, and the FP32 squared
// distance of any candidate within 1.1 h differs from the true one by less
// than 2^-18 h^2.  The band [h^2 (1 - 2^-14), h^2 (1 + 2^-14)] is 16x wider
// than that, and outside the band the reference's test sqrt(fl64(s)) > h
// cannot disagree with the FP32 decision.
#include <algorithm>

#include "sph_cellwarp.cuh"
#include "sph_launch.h"
#include "sphgpu.h"

namespace sphgpu {

namespace {


// The operator bodies on a hit, in FP64 (list entry = q | neighbour cell << 27;
// the force looks up whether q is a wall).
template <int DIM, int OP>
struct Proc64 {
  const State& s;
  const Consts& k;
  double xp[3];
  double vp[3];
  double rhop, prp;
  double acc, ax, ay, az, sx, sy, sz, wp, wg, ws;
  // XSPH: sum_q wx (v_q - v_p) formed as sum_q wx v_q - v_p sum_q wx (the
  // epilogue), the two sums in the neighbour order
  double xw, xv0, xv1, xv2;
  int c0, c1, c2;

  __device__ Proc64(const State& s_, const Consts& k_) : s(s_), k(k_) {
    acc = ax = ay = az = sx = sy = sz = wp = wg = ws = 0.0;
    xw = xv0 = xv1 = xv2 = 0.0;
    rhop = prp = 0.0;
    vp[0] = vp[1] = vp[2] = 0.0;
    c0 = c1 = c2 = 0;
  }

  __device__ __forceinline__ int entry(int q, int c, int tq) const {
    if (OP == SPH_OP_WALL_PRESSURE && tq != kFluid) return kCwSkip;
    return q | (c << kCwCellBits);
  }

  __device__ __forceinline__ void process(const int* list, int stride, int cnt) {
    for (int j = 0; j < cnt; ++j) {
      const int e = __ldg(&list[(size_t)j * stride]);
      if (e == kCwSkip) continue;  // a band candidate beyond the support
      const int q = e & kCwIndexMask;
      double d[3];
      const double r = kdist64<DIM>(s, xp, q, d);
      const bool fluid = OP != SPH_OP_FORCE || __ldg(&s.type[q]) == kFluid;
      if (fluid) ++c0; else ++c1;
      // kernel pieces in the oracle's order (ker_w / ker_rdw), mass folded
      // into the constants, the force sums with fused multiply-adds
      const double t = ker_t(k, r);
      const double t2 = t * t;
      if (OP == SPH_OP_DENSITY || OP == SPH_OP_DENSITY_REF) {
        acc = acc + (t2 * t2) * __fma_rn(k.mcw4, t, k.mcw5);
      } else if (OP == SPH_OP_WALL_PRESSURE) {
        // Adami, Hu & Adams (2012) wall pressure, g . (x_w - x_f)
        const double w = (k.cw * (t2 * t2)) * __fma_rn(-4.0, t, 5.0);
        double gd = __fma_rn(k.g[1], d[1], k.g[0] * d[0]);
        if (DIM == 3) gd = __fma_rn(k.g[2], d[2], gd);
        wp = __fma_rn(__ldg(&s.P[q]), w, wp);
        wg = __fma_rn(__ldg(&s.rho[q]) * gd, w, wg);
        ws = ws + w;
      } else if (fluid) {
        // pressure (collapse_symplectic.jl:114-118) + Monaghan viscosity + XSPH
        const double ker = k.mcr * (t2 * t);
        double vq[3];
        vq[0] = __ldg(&s.v[0][q]);
        vq[1] = __ldg(&s.v[1][q]);
        vq[2] = DIM == 3 ? __ldg(&s.v[2][q]) : 0.0;
        const double dv0 = vp[0] - vq[0];
        const double dv1 = vp[1] - vq[1];
        const double dv2 = DIM == 3 ? vp[2] - vq[2] : 0.0;
        double vdx = __fma_rn(dv1, d[1], dv0 * d[0]);
        if (DIM == 3) vdx = __fma_rn(dv2, d[2], vdx);
        const double rhoq = __ldg(&s.rho[q]);
        const double inv_rb = two_over(rhop + rhoq);
        double pi = 0.0;
        if (lt0(vdx)) {
          // mu = h v.x / (r^2 + eta^2), r^2 + eta^2 as one fused multiply-add,
          // the quotient as a product with the reciprocal
          pi = ((k.ca * vdx) * __drcp_rn(__fma_rn(r, r, k.eta2))) * inv_rb;
          ++c2;
        }
        const double cf = -ker * ((prp + __ldg(&s.Pr[q])) + pi);
        ax = __fma_rn(cf, d[0], ax);
        ay = __fma_rn(cf, d[1], ay);
        if (DIM == 3) az = __fma_rn(cf, d[2], az);
        const double wx = ((t2 * t2) * __fma_rn(k.mcw4, t, k.mcw5)) * inv_rb;
        xw = xw + wx;
        xv0 = __fma_rn(wx, vq[0], xv0);
        xv1 = __fma_rn(wx, vq[1], xv1);
        if (DIM == 3) xv2 = __fma_rn(wx, vq[2], xv2);
      } else {
        // wall neighbour: pressure term with the wall pressure
        const double ker = k.mcr * (t2 * t);
        const double cf = -ker * (prp + __ldg(&s.Pr[q]));
        ax = __fma_rn(cf, d[0], ax);
        ay = __fma_rn(cf, d[1], ay);
        if (DIM == 3) az = __fma_rn(cf, d[2], az);
      }
    }
  }

  // Sums target i's row (sph_tile64.cu wrote each entry's m W and distance,
  // or its pressure and XSPH factors, once per pair): the same terms,
  // accumulated in the same order, as process() over the traversal's list.
  __device__ __forceinline__ void rows(const BinScratch& b, int i, int cnt) {
    const RowEntry* row = b.rows + 4 * (size_t)__ldg(&b.row_base[i]);
    if (OP == SPH_OP_DENSITY || OP == SPH_OP_DENSITY_REF) {
      for (int j = 0; j < cnt; ++j) acc = acc + __ldg(&row[j].a);
      c0 += cnt;
    } else if (OP == SPH_OP_WALL_PRESSURE) {
      // a wall's row: its fluid neighbours with the kernel value W(r) (no
      // mass) and g.(x_w - x_q), both formed by the density pass's pair
      // kernel in the same expressions as process() forms them
      const int n = *b.d_n;
      for (int j = 0; j < cnt; ++j) {
        const RowEntry en = row_load(row + j);
        const int q = (int)(en.q & 0x7fffffffu);
        if (q >= n) {  // an entry the tile passes did not write: report, skip
          atomicOr(b.d_err, kErrBounds);
          continue;
        }
        const double w = en.a, gd = en.b;
        wp = __fma_rn(__ldg(&s.P[q]), w, wp);
        wg = __fma_rn(__ldg(&s.rho[q]) * gd, w, wg);
        ws = ws + w;
      }
      c0 += cnt;
    } else if (OP == SPH_OP_FORCE) {
      const int n = *b.d_n;
      // the separations from the fixed-point copies (exact, integer pipes)
      const long long X0 = b.xfix[0][i], X1 = b.xfix[1][i];
      const long long X2 = DIM == 3 ? b.xfix[2][i] : 0;
      for (int j = 0; j < cnt; ++j) {
        const RowEntry en = row_load(row + j);
        const unsigned long long e = en.q;
        const double cf = en.a, wx = en.b;
        const int q = (int)(e & 0x7fffffffu);
        if (q >= n) {  // an entry the tile passes did not write: report, skip
          atomicOr(b.d_err, kErrBounds);
          continue;
        }
        // q's force record (sph_tile64.cu built it before this pass)
        long long QX0, QX1, QX2;
        double qv0;
        frec_load_x(b.frec + q, QX0, QX1, QX2, qv0);
        const double d0 = fx_sep2(X0, &s.x[0][i], QX0, &s.x[0][q], k.fx_k);
        const double d1 = fx_sep2(X1, &s.x[1][i], QX1, &s.x[1][q], k.fx_k);
        ax = __fma_rn(cf, d0, ax);
        ay = __fma_rn(cf, d1, ay);
        if (DIM == 3) az = __fma_rn(cf, fx_sep2(X2, &s.x[2][i], QX2, &s.x[2][q], k.fx_k), az);
        if ((e & 0x80000000u) == 0u) {
          // fluid neighbour: wx and wx v_q into the XSPH sums
          double qv1, qv2;
          frec_load_v12(b.frec + q, qv1, qv2);
          xw = xw + wx;
          xv0 = __fma_rn(wx, qv0, xv0);
          xv1 = __fma_rn(wx, qv1, xv1);
          if (DIM == 3) xv2 = __fma_rn(wx, qv2, xv2);
          ++c0;
        } else {
          ++c1;
        }
      }
    }
  }
};

// A target's accumulators start at the stored value (apply! accumulates) or
// at 0; the force also needs the target's own velocity, density and P/rho^2.
template <int DIM, int OP>
__device__ __forceinline__ void target_prologue(const State& s, int i, int reset,
                                                Proc64<DIM, OP>& p) {
  if (OP == SPH_OP_DENSITY) {
    if (!reset) p.acc = s.rho[i];
  } else if (OP == SPH_OP_DENSITY_REF) {
    if (!reset) p.acc = s.rho_ref[i];
  } else if (OP == SPH_OP_FORCE) {
    if (!reset) {
      p.ax = s.a[0][i]; p.ay = s.a[1][i];
      p.sx = s.xs[0][i]; p.sy = s.xs[1][i];
      if (DIM == 3) { p.az = s.a[2][i]; p.sz = s.xs[2][i]; }
    }
#pragma unroll
    for (int d = 0; d < DIM; ++d) p.vp[d] = s.v[d][i];
    p.rhop = s.rho[i];
    p.prp = s.Pr[i];
  }
}

// A folded reset_*! still zeroes the targets the operator skips.
template <int DIM, int OP>
__device__ __forceinline__ void skipped_target(const State& s, int i, int reset) {
  if (!reset) return;
  if (OP == SPH_OP_DENSITY) {
    s.rho[i] = 0.0;
  } else if (OP == SPH_OP_DENSITY_REF) {
    s.rho_ref[i] = 0.0;
  } else if (OP == SPH_OP_FORCE) {
#pragma unroll
    for (int d = 0; d < DIM; ++d) { s.a[d][i] = 0.0; s.xs[d][i] = 0.0; }
  }
}

// The epilogue of an acted-on target: self term (core.jl:155-157), fused
// EOS, stores.
template <int DIM, int OP>
__device__ __forceinline__ void target_epilogue(const State& s, const Consts& k, int i,
                                                const Proc64<DIM, OP>& p, int self, int fuse_eos) {
  if (OP == SPH_OP_DENSITY || OP == SPH_OP_DENSITY_REF) {
    double acc = p.acc;
    if (self) acc = acc + k.mass * ker_w(k, 0.0);
    if (OP == SPH_OP_DENSITY) {
      s.rho[i] = acc;
      if (fuse_eos) {
        double P, Pr;
        eos_eval(k, acc, s.rho_ref[i], P, Pr);
        s.P[i] = P;
        s.Pr[i] = Pr;
      }
    } else {
      s.rho_ref[i] = acc;
    }
  } else if (OP == SPH_OP_WALL_PRESSURE) {
    const double P = p.ws > 0.0 ? (p.wp + p.wg) / p.ws : 0.0;
    s.P[i] = P;
    s.Pr[i] = P / (k.rho0 * k.rho0);
    s.rho[i] = k.rho0;
  } else {
    double ax = p.ax, ay = p.ay, az = p.az;
    double sx = p.sx + __fma_rn(-p.vp[0], p.xw, p.xv0);
    double sy = p.sy + __fma_rn(-p.vp[1], p.xw, p.xv1);
    double sz = DIM == 3 ? p.sz + __fma_rn(-p.vp[2], p.xw, p.xv2) : p.sz;
    if (self) {
      const double ker = k.mass * ker_rdw(k, 0.0);
      const double inv_rb = 2.0 / (p.rhop + p.rhop);
      const double cf = -ker * ((p.prp + p.prp) + 0.0);
      const double wx = (k.mass * ker_w(k, 0.0)) * inv_rb;
      ax = ax + cf * 0.0;
      ay = ay + cf * 0.0;
      az = az + cf * 0.0;
      sx = sx + wx * (p.vp[0] - p.vp[0]);
      sy = sy + wx * (p.vp[1] - p.vp[1]);
      sz = sz + wx * (p.vp[2] - p.vp[2]);
    }
    s.a[0][i] = ax;
    s.a[1][i] = ay;
    s.xs[0][i] = sx;
    s.xs[1][i] = sy;
    if (DIM == 3) {
      s.a[2][i] = az;
      s.xs[2][i] = sz;
    }
  }
}

// A persistent grid of at most trav_slots warps, each with its own slot of
// the traversal scratch, taking work items from a counter (zeroed before the
// launch) so that uneven items balance; one warp per item.
template <int DIM, int OP, int WARPS>
__global__ void __launch_bounds__(32 * WARPS) pair64_kernel(State s, Geometry g, Consts k,
                                                            BinScratch b, int self, int reset,
                                                            int fuse_eos, int list_mode) {
  __shared__ CwShared shared[WARPS];
  const int lane = threadIdx.x & 31;
  const int w = threadIdx.x >> 5;
  const int slot = blockIdx.x * WARPS + w;
  if (slot >= b.trav_slots) return;  // warp-uniform
  // list_mode 3: the row sums took every target whose row is complete;
  // only overflowed rows traverse here
  if (list_mode == 3 && *b.d_rover == 0 && *b.d_pover == 0) return;
  const int total = __ldg(&b.item_off[g.key_max + 1]);
  // the wall pressure acts on wall targets, every other operator on fluid ones
  const int want = OP == SPH_OP_WALL_PRESSURE ? kWall : kFluid;
  for (;;) {
    int item = 0;
    if (lane == 0) item = atomicAdd(b.work_ctr, 1);
    item = __shfl_sync(0xffffffffu, item, 0);
    if (item >= total) break;
    const int2 it = __ldg(&b.items[item]);
    const int first = it.x, count = it.y;
    const int i = first + lane;
    const bool valid = lane < count;
    const int ti = valid ? s.type[i] : -1;
    CwTarget t;
    t.active = valid && ti == want;
    if (list_mode == 3)
      t.active = t.active && (__ldg(&b.hit_count[i]) == kRowOver || *b.d_pover != 0);
    else if (valid && ti != want)
      skipped_target<DIM, OP>(s, i, reset);
    // an item without targets of the operator has nothing to traverse
    if (!__any_sync(0xffffffffu, t.active)) continue;
    t.i = i;
    t.key = s.cell[first];
    decode_key(g, t.key, t.cx, t.cy, t.cz);
    t.pi4 = valid ? s.pl[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    t.xp[0] = valid ? s.x[0][i] : 0.0;
    t.xp[1] = valid ? s.x[1][i] : 0.0;
    t.xp[2] = (DIM == 3 && valid) ? s.x[2][i] : 0.0;
    Proc64<DIM, OP> p(s, k);
    p.xp[0] = t.xp[0];
    p.xp[1] = t.xp[1];
    p.xp[2] = t.xp[2];
    if (t.active) target_prologue<DIM, OP>(s, i, reset, p);
    cw_pass<DIM, OP>(s, g, k, b, shared[w], lane, t, p, slot);
    if (t.active) target_epilogue<DIM, OP>(s, k, i, p, self, fuse_eos);
    cw_count<OP>(b, p.c0, p.c1, p.c2);
  }
}

// The density, wall-pressure and force passes of a step over the rows the
// tile passes wrote (sph_tile64.cu): one thread per particle; targets whose
// rows overflowed are left to pair64_kernel.
template <int DIM, int OP>
__global__ void __launch_bounds__(256, 5) row_sum_kernel(State s, Consts k, BinScratch b, int self,
                                                      int reset, int fuse_eos) {
  const int n = *b.d_n;
  const int i = blockIdx.x * 256 + threadIdx.x;
  // the wall pressure acts on wall targets, every other operator on fluid ones
  const int want = OP == SPH_OP_WALL_PRESSURE ? kWall : kFluid;
  Proc64<DIM, OP> p(s, k);
  if (i < n) {
    if (s.type[i] != want) {
      skipped_target<DIM, OP>(s, i, reset);
    } else {
      const int cnt = __ldg(&b.hit_count[i]);
      if (cnt != kRowOver && *b.d_pover == 0) {
        p.xp[0] = s.x[0][i];
        p.xp[1] = s.x[1][i];
        p.xp[2] = DIM == 3 ? s.x[2][i] : 0.0;
        target_prologue<DIM, OP>(s, i, reset, p);
        p.rows(b, i, cnt);
        target_epilogue<DIM, OP>(s, k, i, p, self, fuse_eos);
      }
    }
  }
  cw_count<OP>(b, p.c0, p.c1, p.c2);
}

// The wall pressure of a step over the walls' rows (their fluid neighbours,
// written by the density pass): one thread per wall, taken from the lists
// the row count made -- threads [0, A) the A walls with fluid neighbours (so
// every lane of a warp has a row to sum: the FP64 pipe, GB300's scarcest,
// issues only for walls with work), threads [A, A + B) the walls without,
// which get the empty sum (P = 0).  Each sum runs over the wall's row in its
// order -- the reference's summation order, as Proc64::rows forms it.  Walls
// whose rows are not used (kRowOver, or every target after an overflow) are
// left to pair64_kernel.
template <int DIM>
__global__ void __launch_bounds__(256) wall_rows_kernel(State s, Consts k, BinScratch b) {
  if (*b.d_pover) return;  // every wall traverses
  const int na = b.d_nwall[0], nb = b.d_nwall[1];
  const int t = blockIdx.x * 256 + threadIdx.x;
  int c0 = 0;
  if (t < na) {
    const int i = b.wall_list[t];
    const int cnt = __ldg(&b.hit_count[i]);
    Proc64<DIM, SPH_OP_WALL_PRESSURE> p(s, k);
    p.rows(b, i, cnt);
    target_epilogue<DIM, SPH_OP_WALL_PRESSURE>(s, k, i, p, 0, 0);
    c0 = p.c0;
  } else if (t < na + nb) {
    const int i = b.wall_list[b.wall_cap - 1 - (t - na)];
    s.P[i] = 0.0;
    s.Pr[i] = 0.0 / (k.rho0 * k.rho0);
    s.rho[i] = k.rho0;
  }
  cw_count<SPH_OP_WALL_PRESSURE>(b, c0, 0, 0);
}

// sum(sys, func, x) (core.jl:240-260) / sum(sys, func, p) (core.jl:271-291):
// one thread per query, straight FP64 traversal (self included).
template <int DIM>
__global__ void __launch_bounds__(128) sum_kernel(State s, Geometry g, Consts k, BinScratch b,
                                                  int func, int nq, const double* xq,
                                                  const long long* rid_query, double* out) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nq) return;
  double x[3];
  if (rid_query) {
    const int p = b.inv_rid[rid_query[t]];
    x[0] = s.x[0][p];
    x[1] = s.x[1][p];
    x[2] = DIM == 3 ? s.x[2][p] : 0.0;
  } else {
    x[0] = xq[3 * t];
    x[1] = xq[3 * t + 1];
    x[2] = xq[3 * t + 2];
  }
  const long long key = find_key_point(g, k, x);
  double acc = 0.0;
  for (int c = 0; c < g.n_diff; ++c) {
    const long long nk = key + g.key_diff[c];
    if (!(1 <= nk && nk <= g.key_max)) continue;
    const int st = b.cell_start[nk], en = b.cell_start[nk + 1];
    for (int q = st; q < en; ++q) {
      const double d0 = x[0] - s.x[0][q];
      const double d1 = x[1] - s.x[1][q];
      const double d2 = x[2] - (DIM == 3 ? s.x[2][q] : 0.0);
      const double r = sqrt((d0 * d0 + d1 * d1) + d2 * d2);
      if (r > k.h) continue;
      const int tq = s.type[q];
      double f = 0.0;
      switch (func) {
        case SPH_SUM_DENSITY:
          f = k.mass * ker_w(k, r);
          break;
        case SPH_SUM_KERNEL:
          f = ker_w(k, r);
          break;
        case SPH_SUM_PRESSURE:
          f = tq == kFluid ? ((k.mass / s.rho[q]) * s.P[q]) * ker_w(k, r) : 0.0;
          break;
        case SPH_SUM_SHEPARD:
          f = tq == kFluid ? (k.mass / s.rho[q]) * ker_w(k, r) : 0.0;
          break;
        default:
          break;
      }
      acc = acc + f;
    }
  }
  out[t] = acc;
}

// Every ordered pair within the support, classified exactly as the pair
// passes classify candidates (FP32 with the FP64 band test).
template <int DIM>
__global__ void __launch_bounds__(128) debug_pairs_kernel(State s, Geometry g, Consts k,
                                                          BinScratch b, int pass, int* counts,
                                                          const long long* offsets,
                                                          long long* pairs, long long cap_pairs) {
  const int n = *b.d_n;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int key = s.cell[i];
  int cx, cy, cz;
  decode_key(g, key, cx, cy, cz);
  const float4 pi4 = s.pl[i];
  double xp[3];
  xp[0] = s.x[0][i];
  xp[1] = s.x[1][i];
  xp[2] = DIM == 3 ? s.x[2][i] : 0.0;
  const int rid = s.rid[i];
  long long pos = pass ? offsets[rid] : 0;
  int cnt = 0;
  for (int c = 0; c < g.n_diff; ++c) {
    const int nk = key + g.key_diff[c];
    if (nk < 1 || nk > g.key_max) continue;
    int qx, qy, qz;
    decode_key(g, nk, qx, qy, qz);
    const float ox = (float)(qx - cx) * k.cellf;
    const float oy = (float)(qy - cy) * k.cellf;
    const float oz = (float)(qz - cz) * k.cellf;
    for (int q = b.cell_start[nk]; q < b.cell_start[nk + 1]; ++q) {
      const float4 pq = s.pl[q];
      const float dx = (pi4.x - pq.x) - ox;
      const float dy = (pi4.y - pq.y) - oy;
      float ss = dx * dx + dy * dy;
      if (DIM == 3) {
        const float dz = (pi4.z - pq.z) - oz;
        ss = ss + dz * dz;
      }
      if (ss > k.s_hi || q == i) continue;
      if (!(ss < k.s_lo) && !within_rn<DIM>(s, k, xp, q)) continue;
      if (pass && pos < cap_pairs) {
        pairs[2 * pos] = rid;
        pairs[2 * pos + 1] = s.rid[q];
      }
      ++pos;
      ++cnt;
    }
  }
  if (!pass) counts[rid] = cnt;
}
// The pairs the last density pass acted on, read back from what it stored
// for the pass after it: an FP64 fluid target's row (its neighbours' indices
// in the reference's order) or a mixed-precision target's hit masks, decoded
// chunk by chunk in the traversal order (key_diff order, 32 candidates per
// chunk, bit u = candidate u).  Pass 0 counts per reference index, pass 1
// writes (rid_p, rid_q) at offsets[rid_p].  A fluid target whose hits were not
// stored (an overflowed row, mask slots beyond the capacity) sets *bad.
__global__ void __launch_bounds__(128) debug_hits_kernel(State s, Geometry g, BinScratch b,
                                                         int mixed, int pass, int* counts,
                                                         const long long* offsets,
                                                         long long* pairs, long long cap_pairs,
                                                         int* bad) {
  const int n = *b.d_n;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int rid = s.rid[i];
  long long pos = pass ? offsets[rid] : 0;
  int cnt = 0;
  if (s.type[i] == kFluid) {
    if (!mixed) {
      const int hc = b.hit_count[i];
      if (hc == kRowOver || *b.d_pover != 0) {
        atomicOr(bad, 1);
      } else {
        const RowEntry* row = b.rows + 4 * (size_t)b.row_base[i];
        for (int j = 0; j < hc; ++j, ++pos, ++cnt)
          if (pass && pos < cap_pairs) {
            pairs[2 * pos] = rid;
            pairs[2 * pos + 1] = s.rid[(int)(row[j].q & 0x7fffffffu)];
          }
      }
    } else {
      // the target's work item and lane, and the item's mask slots (the
      // binning counted them per cell: items of a cell x chunks per item)
      const int key = s.cell[i];
      const int local = i - b.cell_start[key];
      const int i0 = b.item_off[key], ni = b.item_off[key + 1] - i0;
      const int item = i0 + (local >> 5), lane = local & 31;
      const int co = b.chunk_off[key];
      const int nc = ni > 0 ? (b.chunk_off[key + 1] - co) / ni : 0;
      const long long start = (long long)co + (long long)(item - i0) * nc;
      if (start + nc > (long long)b.ck_cap) {
        atomicOr(bad, 2);
      } else {
        int gi = 0;
        for (int c = 0; c < g.n_diff; ++c) {
          const int nk = key + g.key_diff[c];
          if (nk < 1 || nk > g.key_max) continue;  // core.jl:98
          const int en = b.cell_start[nk + 1];
          for (int base = b.cell_start[nk]; base < en; base += 32, ++gi) {
            if (gi >= nc) {
              atomicOr(bad, 4);
              break;
            }
            unsigned mask = b.ck_mask[((size_t)start + gi) * 32 + lane];
            while (mask) {
              const int u = __ffs(mask) - 1;
              mask &= mask - 1u;
              if (pass && pos < cap_pairs) {
                pairs[2 * pos] = rid;
                pairs[2 * pos + 1] = s.rid[base + u];
              }
              ++pos;
              ++cnt;
            }
          }
        }
      }
    }
  }
  if (!pass) counts[rid] = cnt;
}

// pair64_kernel: at most one resident wave of blocks and at most
// trav_slots warps (each needs its own slot of the traversal scratch)
template <int DIM, int OP, int WARPS>
void pair64_launch(cudaStream_t st, const BinScratch& b, int threads, const State& s,
                   const Geometry& g, const Consts& k, const BinScratch& bb, int self, int reset,
                   int fuse_eos, int list_mode) {
  static const int wave = resident_blocks(pair64_kernel<DIM, OP, WARPS>, 32 * WARPS);
  const int need = std::max(1, std::min(b.max_items, b.trav_slots));
  const int blocks = std::max(1, std::min((need + WARPS - 1) / WARPS, wave));
  cudaMemsetAsync(b.work_ctr, 0, sizeof(int), st);
  pair64_kernel<DIM, OP, WARPS><<<blocks, threads, 0, st>>>(s, g, k, bb, self, reset, fuse_eos,
                                                           list_mode);
}

template <int DIM>
cudaError_t launch_pair_dim(const LaunchCtx& c, const State& s, const Geometry& g,
                            const Consts& k, const BinScratch& b, int cap, int op, int self,
                            int reset, int fuse_eos, int list_mode) {
  const int W = k.warps;
  const int kid = op == SPH_OP_FORCE           ? SPH_KERNEL_FORCE
                  : op == SPH_OP_WALL_PRESSURE ? SPH_KERNEL_WALL
                                               : SPH_KERNEL_DENSITY;
  mark(c, kid, 0);
  // the density and force passes of a step: every pair evaluated once into
  // the rows (sph_tile64.cu), the rows summed, then the traversal of the
  // targets whose rows overflowed (its warps return at once otherwise)
  if (list_mode == 3) {
    const int rb = (cap + 255) / 256;
    if (op == SPH_OP_WALL_PRESSURE) {
      // the density pass's rows hold every wall's fluid neighbours
      wall_rows_kernel<DIM><<<(cap + 255) / 256, 256, 0, c.stream>>>(s, k, b);
    } else {
      const cudaError_t e = launch_tiles_fp64(c, s, g, k, b, cap, op == SPH_OP_FORCE ? 1 : 0);
      if (e != cudaSuccess) return e;
      if (op == SPH_OP_FORCE)
        row_sum_kernel<DIM, SPH_OP_FORCE><<<rb, 256, 0, c.stream>>>(s, k, b, self, reset, 0);
      else if (op == SPH_OP_DENSITY_REF)
        row_sum_kernel<DIM, SPH_OP_DENSITY_REF><<<rb, 256, 0, c.stream>>>(s, k, b, self, reset, 0);
      else
        row_sum_kernel<DIM, SPH_OP_DENSITY><<<rb, 256, 0, c.stream>>>(s, k, b, self, reset,
                                                                      fuse_eos);
    }
  }
  switch (op) {
    case SPH_OP_DENSITY:
      if (W == 2) pair64_launch<DIM, SPH_OP_DENSITY, 2>(c.stream, b, 64, s, g, k, b, self, reset, fuse_eos, list_mode);
      else if (W == 8) pair64_launch<DIM, SPH_OP_DENSITY, 8>(c.stream, b, 256, s, g, k, b, self, reset, fuse_eos, list_mode);
      else pair64_launch<DIM, SPH_OP_DENSITY, 4>(c.stream, b, 128, s, g, k, b, self, reset, fuse_eos, list_mode);
      break;
    case SPH_OP_DENSITY_REF:
      if (W == 2) pair64_launch<DIM, SPH_OP_DENSITY_REF, 2>(c.stream, b, 64, s, g, k, b, self, reset, 0, list_mode);
      else if (W == 8) pair64_launch<DIM, SPH_OP_DENSITY_REF, 8>(c.stream, b, 256, s, g, k, b, self, reset, 0, list_mode);
      else pair64_launch<DIM, SPH_OP_DENSITY_REF, 4>(c.stream, b, 128, s, g, k, b, self, reset, 0, list_mode);
      break;
    case SPH_OP_WALL_PRESSURE:
      if (W == 2) pair64_launch<DIM, SPH_OP_WALL_PRESSURE, 2>(c.stream, b, 64, s, g, k, b, 0, 0, 0, list_mode);
      else if (W == 8) pair64_launch<DIM, SPH_OP_WALL_PRESSURE, 8>(c.stream, b, 256, s, g, k, b, 0, 0, 0, list_mode);
      else pair64_launch<DIM, SPH_OP_WALL_PRESSURE, 4>(c.stream, b, 128, s, g, k, b, 0, 0, 0, list_mode);
      break;
    default:
      if (W == 2) pair64_launch<DIM, SPH_OP_FORCE, 2>(c.stream, b, 64, s, g, k, b, self, reset, 0, list_mode);
      else if (W == 8) pair64_launch<DIM, SPH_OP_FORCE, 8>(c.stream, b, 256, s, g, k, b, self, reset, 0, list_mode);
      else pair64_launch<DIM, SPH_OP_FORCE, 4>(c.stream, b, 128, s, g, k, b, self, reset, 0, list_mode);
      break;
  }
  mark(c, kid, 1,
       list_mode != 3                 ? 1
       : op == SPH_OP_WALL_PRESSURE ? 2
                                    : kRowPassLaunches[op == SPH_OP_FORCE ? 1 : 0]);
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_pair_fp64(const LaunchCtx& c, const State& s, const Geometry& g,
                             const Consts& k, const BinScratch& b, int cap, int op, int self,
                             int reset, int fuse_eos, int lists_valid) {
  if (cap <= 0) return cudaSuccess;
  // rows: the density passes (rho and the reference density) always build
  // them; the wall-pressure and force passes sum them when a density pass of
  // this binning built them, else they traverse
  const int lm = op == SPH_OP_DENSITY || op == SPH_OP_DENSITY_REF ||
                         ((op == SPH_OP_FORCE || op == SPH_OP_WALL_PRESSURE) && lists_valid)
                     ? 3
                     : 0;
  return k.dim == 2 ? launch_pair_dim<2>(c, s, g, k, b, cap, op, self, reset, fuse_eos, lm)
                    : launch_pair_dim<3>(c, s, g, k, b, cap, op, self, reset, fuse_eos, lm);
}

cudaError_t launch_sum(const LaunchCtx& c, const State& s, const Geometry& g, const Consts& k,
                       const BinScratch& b, int func, int nq, const double* x,
                       const long long* rid_query, double* out) {
  if (nq <= 0) return cudaSuccess;
  const int blocks = (nq + 127) / 128;
  mark(c, SPH_KERNEL_SUM, 0);
  if (k.dim == 2)
    sum_kernel<2><<<blocks, 128, 0, c.stream>>>(s, g, k, b, func, nq, x, rid_query, out);
  else
    sum_kernel<3><<<blocks, 128, 0, c.stream>>>(s, g, k, b, func, nq, x, rid_query, out);
  mark(c, SPH_KERNEL_SUM, 1);
  return cudaGetLastError();
}

cudaError_t launch_debug_hits(const LaunchCtx& c, const State& s, const Geometry& g,
                              const BinScratch& b, int cap, int mixed, int pass, int* counts,
                              const long long* offsets, long long* pairs, long long cap_pairs,
                              int* bad) {
  if (cap <= 0) return cudaSuccess;
  mark(c, SPH_KERNEL_SUM, 0);
  debug_hits_kernel<<<(cap + 127) / 128, 128, 0, c.stream>>>(s, g, b, mixed, pass, counts, offsets,
                                                              pairs, cap_pairs, bad);
  mark(c, SPH_KERNEL_SUM, 1);
  return cudaGetLastError();
}

cudaError_t launch_debug_pairs(const LaunchCtx& c, const State& s, const Geometry& g,
                               const Consts& k, const BinScratch& b, int cap, int pass,
                               int* counts, const long long* offsets, long long* pairs,
                               long long cap_pairs) {
  if (cap <= 0) return cudaSuccess;
  const int blocks = (cap + 127) / 128;
  mark(c, SPH_KERNEL_SUM, 0);
  if (k.dim == 2)
    debug_pairs_kernel<2><<<blocks, 128, 0, c.stream>>>(s, g, k, b, pass, counts, offsets, pairs, cap_pairs);
  else
    debug_pairs_kernel<3><<<blocks, 128, 0, c.stream>>>(s, g, k, b, pass, counts, offsets, pairs, cap_pairs);
  mark(c, SPH_KERNEL_SUM, 1);
  return cudaGetLastError();
}

}  // namespace sphgpu
