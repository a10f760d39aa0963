// sph_pair64.cu -- the FP64 pair passes: _apply_binary! (core.jl:94-112) for
// the built-in operators, sum(sys, func, x / p) (core.jl:240-291) and the
// neighbour-pair listing used by the parity tests.
//
// Built with --fmad=false: every FP64 expression rounds exactly where it is
// written, in the order the CPU restatement uses, so results are bit-identical
// to it (IEEE division and square root are correctly rounded on both sides).
//
// Pair pass structure (one thread per target particle, targets in cell order,
// so the lanes of a warp mostly share one cell and walk the same candidates):
//   scan    : walk the 3^d neighbour cells in key_diff order and each cell's
//             particles in stored (descending reference index) order.  Each
//             candidate is classified with FP32 arithmetic on cell-relative
//             positions; only candidates inside a thin band around the
//             support radius are re-tested with the reference's FP64
//             expression.  Hits go to a per-thread queue in shared memory.
//   process : the queued hits are evaluated in FP64, in queue order, so each
//             target's sums are formed in exactly the reference's order.
// The FP64 pipe is the bound of this pass (1/58 of the FP32 rate on GB300),
// and the split keeps every FP64 instruction on a hit with the warp's lanes
// busy, instead of one FP64 distance per candidate.
//
// Why the FP32 classification is exact: positions are stored relative to
// their cell's origin, |xl| < 1.02 h; the neighbour-cell offset is an integer
// multiple of fl32(h).  Each component of the FP32 separation then differs
// from the true separation by at most 8 * 2^-24 h, so the FP32 squared
// distance of any candidate within 1.1 h differs from the true one by less
// than 2^-18 h^2.  The band [h^2 (1 - 2^-14), h^2 (1 + 2^-14)] is 16x wider
// than that, and outside the band the reference's test sqrt(fl64(s)) > h
// cannot disagree with the FP32 decision.
#include "sph_launch.h"
#include "sphgpu.h"

namespace sphgpu {

namespace {

constexpr int kPairThreads = 128;
constexpr int kQueue = 32;

template <int DIM>
__device__ __forceinline__ double dist2_64(const State& s, const double* xp, int q, double* d) {
  d[0] = xp[0] - __ldg(&s.x[0][q]);
  d[1] = xp[1] - __ldg(&s.x[1][q]);
  double ss = d[0] * d[0] + d[1] * d[1];
  if (DIM == 3) {
    d[2] = xp[2] - __ldg(&s.x[2][q]);
    ss = ss + d[2] * d[2];
  } else {
    d[2] = 0.0;
  }
  return ss;
}

__device__ __forceinline__ void warp_add(unsigned long long* dst, int v) {
  const int sum = __reduce_add_sync(0xffffffffu, v);
  if ((threadIdx.x & 31) == 0 && sum) atomicAdd(dst, (unsigned long long)sum);
}

// Pair and per-category hit counters (c0: the operator's main hits; for the
// force c0 = fluid neighbours, c1 = wall neighbours, c2 = viscosity active).
template <int OP>
__device__ __forceinline__ void count_hits(const BinScratch& b, int pairs, int c0, int c1, int c2) {
  warp_add(b.d_pairs, pairs);
  if (OP == SPH_OP_FORCE) {
    warp_add(b.d_cat + kCatForceFluid, c0);
    warp_add(b.d_cat + kCatForceWall, c1);
    warp_add(b.d_cat + kCatForceAV, c2);
  } else if (OP == SPH_OP_WALL_PRESSURE) {
    warp_add(b.d_cat + kCatWall, c0);
  } else {
    warp_add(b.d_cat + kCatDensity, c0);
  }
}

template <int DIM, int OP>
__global__ void __launch_bounds__(kPairThreads) pair64_kernel(State s, Geometry g, Consts k,
                                                              BinScratch b, int self, int reset,
                                                              int fuse_eos) {
  __shared__ int queue[kQueue][kPairThreads];
  const int tid = threadIdx.x;
  const int n = *b.d_n;
  const int i = blockIdx.x * kPairThreads + tid;
  // the wall pressure acts on wall targets, every other operator on fluid ones
  const int want = OP == SPH_OP_WALL_PRESSURE ? kWall : kFluid;
  int pairs = 0, c0 = 0, c1 = 0, c2 = 0;
  if (i < n && s.type[i] != want) {
    // a folded reset_*! still zeroes the targets the operator skips
    if (reset) {
      if (OP == SPH_OP_DENSITY) {
        s.rho[i] = 0.0;
      } else if (OP == SPH_OP_DENSITY_REF) {
        s.rho_ref[i] = 0.0;
      } else if (OP == SPH_OP_FORCE) {
#pragma unroll
        for (int d = 0; d < DIM; ++d) { s.a[d][i] = 0.0; s.xs[d][i] = 0.0; }
      }
    }
  } else if (i < n) {
    const int key = s.cell[i];
    int cx, cy, cz;
    decode_key(g, key, cx, cy, cz);
    const float4 pi4 = s.pl[i];
    double xp[3];
    xp[0] = s.x[0][i];
    xp[1] = s.x[1][i];
    xp[2] = DIM == 3 ? s.x[2][i] : 0.0;
    // accumulators start at the stored value (apply! accumulates) or at 0
    double acc = 0.0;
    double ax = 0.0, ay = 0.0, az = 0.0, sx = 0.0, sy = 0.0, sz = 0.0;
    double wp = 0.0, wg = 0.0, ws = 0.0;
    double vp[3] = {0.0, 0.0, 0.0};
    double rhop = 0.0, prp = 0.0;
    if (OP == SPH_OP_DENSITY) {
      if (!reset) acc = s.rho[i];
    } else if (OP == SPH_OP_DENSITY_REF) {
      if (!reset) acc = s.rho_ref[i];
    } else if (OP == SPH_OP_FORCE) {
      if (!reset) {
        ax = s.a[0][i]; ay = s.a[1][i];
        sx = s.xs[0][i]; sy = s.xs[1][i];
        if (DIM == 3) { az = s.a[2][i]; sz = s.xs[2][i]; }
      }
#pragma unroll
      for (int d = 0; d < DIM; ++d) vp[d] = s.v[d][i];
      rhop = s.rho[i];
      prp = s.Pr[i];
    }

    int c = 0, j = 0, jend = 0;
    float ox = 0.f, oy = 0.f, oz = 0.f;
    bool more = true;
    while (more) {
      // ---- scan: fill this thread's queue
      int cnt = 0;
      while (cnt < kQueue) {
        if (j >= jend) {
          if (c >= g.n_diff) { more = false; break; }
          const int nk = key + g.key_diff[c];
          ++c;
          if (nk < 1 || nk > g.key_max) continue;  // core.jl:98
          j = __ldg(&b.cell_start[nk]);
          jend = __ldg(&b.cell_start[nk + 1]);
          int qx, qy, qz;
          decode_key(g, nk, qx, qy, qz);
          ox = (float)(qx - cx) * k.hf;
          oy = (float)(qy - cy) * k.hf;
          oz = (float)(qz - cz) * k.hf;
          continue;
        }
        const int q = j++;
        const float4 pq = __ldg(&s.pl[q]);
        const float dx = (pi4.x - pq.x) - ox;
        const float dy = (pi4.y - pq.y) - oy;
        float ss = dx * dx + dy * dy;
        if (DIM == 3) {
          const float dz = (pi4.z - pq.z) - oz;
          ss = ss + dz * dz;
        }
        if (ss > k.s_hi || q == i) continue;
        if (!(ss < k.s_lo) && !within_rn<DIM>(s, k, xp, q)) continue;
        ++pairs;
        const int tq = __float_as_int(pq.w);
        if (OP == SPH_OP_WALL_PRESSURE) {
          if (tq == kFluid) queue[cnt++][tid] = q;
        } else if (OP == SPH_OP_FORCE) {
          queue[cnt++][tid] = tq == kFluid ? q : -q - 1;
        } else {
          queue[cnt++][tid] = q;
        }
      }
      // ---- process: FP64, in queue (= reference) order
      for (int t = 0; t < cnt; ++t) {
        const int e = queue[t][tid];
        const int q = e >= 0 ? e : -e - 1;
        double d[3];
        const double ss = dist2_64<DIM>(s, xp, q, d);
        const double r = sqrt(ss);
        if (e >= 0) ++c0; else ++c1;
        if (OP == SPH_OP_DENSITY || OP == SPH_OP_DENSITY_REF) {
          acc = acc + k.mass * ker_w(k, r);
        } else if (OP == SPH_OP_WALL_PRESSURE) {
          const double w = ker_w(k, r);
          double gd = k.g[0] * d[0] + k.g[1] * d[1];
          if (DIM == 3) gd = gd + k.g[2] * d[2];
          wp = wp + __ldg(&s.P[q]) * w;
          wg = wg + (__ldg(&s.rho[q]) * gd) * w;
          ws = ws + w;
        } else if (e >= 0) {
          // pressure (collapse_symplectic.jl:114-118) + Monaghan viscosity + XSPH
          const double ker = k.mass * ker_rdw(k, r);
          double vq[3];
          vq[0] = __ldg(&s.v[0][q]);
          vq[1] = __ldg(&s.v[1][q]);
          vq[2] = DIM == 3 ? __ldg(&s.v[2][q]) : 0.0;
          const double dv0 = vp[0] - vq[0];
          const double dv1 = vp[1] - vq[1];
          double vdx = dv0 * d[0] + dv1 * d[1];
          if (DIM == 3) {
            const double dv2 = vp[2] - vq[2];
            vdx = vdx + dv2 * d[2];
          }
          const double rhoq = __ldg(&s.rho[q]);
          const double inv_rb = 2.0 / (rhop + rhoq);
          double pi = 0.0;
          if (vdx < 0.0) {
            const double mu = (k.h_smooth * vdx) / (ss + k.eta2);
            pi = (-k.alpha_c0 * mu) * inv_rb;
            ++c2;
          }
          const double cf = -ker * ((prp + __ldg(&s.Pr[q])) + pi);
          ax = ax + cf * d[0];
          ay = ay + cf * d[1];
          if (DIM == 3) az = az + cf * d[2];
          const double wx = (k.mass * ker_w(k, r)) * inv_rb;
          sx = sx + wx * (vq[0] - vp[0]);
          sy = sy + wx * (vq[1] - vp[1]);
          if (DIM == 3) sz = sz + wx * (vq[2] - vp[2]);
        } else {
          // wall neighbour: pressure term with the wall pressure
          const double ker = k.mass * ker_rdw(k, r);
          const double cf = -ker * (prp + __ldg(&s.Pr[q]));
          ax = ax + cf * d[0];
          ay = ay + cf * d[1];
          if (DIM == 3) az = az + cf * d[2];
        }
      }
    }
    // ---- epilogue: self term (core.jl:155-157), fused EOS, stores
    if (OP == SPH_OP_DENSITY || OP == SPH_OP_DENSITY_REF) {
      if (self) acc = acc + k.mass * ker_w(k, 0.0);
      if (OP == SPH_OP_DENSITY) {
        s.rho[i] = acc;
        if (fuse_eos) {
          const double ratio = acc / s.rho_ref[i];
          const double r2 = ratio * ratio;
          const double r4 = r2 * r2;
          const double r7 = (r4 * r2) * ratio;
          const double P = k.B * (r7 - 1.0);
          s.P[i] = P;
          s.Pr[i] = P / (acc * acc);
        }
      } else {
        s.rho_ref[i] = acc;
      }
    } else if (OP == SPH_OP_WALL_PRESSURE) {
      const double P = ws > 0.0 ? (wp + wg) / ws : 0.0;
      s.P[i] = P;
      s.Pr[i] = P / (k.rho0 * k.rho0);
      s.rho[i] = k.rho0;
    } else {
      if (self) {
        const double ker = k.mass * ker_rdw(k, 0.0);
        const double inv_rb = 2.0 / (rhop + rhop);
        const double cf = -ker * ((prp + prp) + 0.0);
        const double wx = (k.mass * ker_w(k, 0.0)) * inv_rb;
        ax = ax + cf * 0.0;
        ay = ay + cf * 0.0;
        az = az + cf * 0.0;
        sx = sx + wx * (vp[0] - vp[0]);
        sy = sy + wx * (vp[1] - vp[1]);
        sz = sz + wx * (vp[2] - vp[2]);
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
  count_hits<OP>(b, pairs, c0, c1, c2);
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
    const float ox = (float)(qx - cx) * k.hf;
    const float oy = (float)(qy - cy) * k.hf;
    const float oz = (float)(qz - cz) * k.hf;
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

template <int DIM>
cudaError_t launch_pair_dim(const LaunchCtx& c, const State& s, const Geometry& g,
                            const Consts& k, const BinScratch& b, int cap, int op, int self,
                            int reset, int fuse_eos) {
  const int blocks = (cap + kPairThreads - 1) / kPairThreads;
  const int kid = op == SPH_OP_FORCE           ? SPH_KERNEL_FORCE
                  : op == SPH_OP_WALL_PRESSURE ? SPH_KERNEL_WALL
                                               : SPH_KERNEL_DENSITY;
  mark(c, kid, 0);
  switch (op) {
    case SPH_OP_DENSITY:
      pair64_kernel<DIM, SPH_OP_DENSITY><<<blocks, kPairThreads, 0, c.stream>>>(s, g, k, b, self, reset, fuse_eos);
      break;
    case SPH_OP_DENSITY_REF:
      pair64_kernel<DIM, SPH_OP_DENSITY_REF><<<blocks, kPairThreads, 0, c.stream>>>(s, g, k, b, self, reset, 0);
      break;
    case SPH_OP_WALL_PRESSURE:
      pair64_kernel<DIM, SPH_OP_WALL_PRESSURE><<<blocks, kPairThreads, 0, c.stream>>>(s, g, k, b, 0, 0, 0);
      break;
    default:
      pair64_kernel<DIM, SPH_OP_FORCE><<<blocks, kPairThreads, 0, c.stream>>>(s, g, k, b, self, reset, 0);
      break;
  }
  mark(c, kid, 1);
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_pair_fp64(const LaunchCtx& c, const State& s, const Geometry& g,
                             const Consts& k, const BinScratch& b, int cap, int op, int self,
                             int reset, int fuse_eos) {
  if (cap <= 0) return cudaSuccess;
  return k.dim == 2 ? launch_pair_dim<2>(c, s, g, k, b, cap, op, self, reset, fuse_eos)
                    : launch_pair_dim<3>(c, s, g, k, b, cap, op, self, reset, fuse_eos);
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
