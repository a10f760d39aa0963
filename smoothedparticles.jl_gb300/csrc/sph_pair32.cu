// sph_pair32.cu -- mixed-precision pair passes.
//
// Same traversal and the same candidate classification as the FP64 passes
// (FP32 test on cell-relative positions, FP64 band test with round-to-nearest
// intrinsics), so the set of pairs is identical to the FP64 path for the same
// positions.  What changes is the arithmetic on a hit:
//   * the separation is the FP32 cell-relative one the scan tested (x_p - x_q
//     with both positions within one cell of their origins, accurate to
//     ~2^-21 h), rebuilt from the hit's index and neighbour-cell number;
//   * kernel values, pressure, viscosity and XSPH terms are FP32, with the
//     neighbour's (v, P/rho^2, rho) read from a 20-byte FP32 copy;
//   * each queue batch (<= 32 hits) is summed in FP32 and folded into FP64
//     accumulators, so FP64 adds are per batch, not per hit;
//   * positions, the self term, the EOS, the wall-pressure quotient and the
//     time integration stay FP64.
// Built with FMA contraction (the FP64 band test uses explicit intrinsics).
#include "sph_cellwarp.cuh"
#include "sph_launch.h"
#include "sphgpu.h"

namespace sphgpu {

namespace {


// FP32 Wendland quintic pieces: t = 1 - r/h (0 outside the support)
__device__ __forceinline__ float kt32(const Consts& k, float r) {
  const float x = r * k.inv_hf;
  return x > 1.f ? 0.f : 1.f - x;
}
__device__ __forceinline__ float kw32(const Consts& k, float r, float t) {
  const float t2 = t * t;
  return k.cwf * (t2 * t2) * (5.f - 4.f * t);  // 1 + 4x = 5 - 4t
}
__device__ __forceinline__ float krdw32(const Consts& k, float t) { return k.crf * (t * t * t); }

__device__ __forceinline__ float fsqrt(float ss) { return ss > 0.f ? ss * rsqrtf(ss) : 0.f; }

template <int DIM>
__global__ void __launch_bounds__(256) aux_refresh_kernel(State s, BinScratch b) {
  const int n = *b.d_n;
  const int i = blockIdx.x * 256 + threadIdx.x;
  if (i >= n) return;
  s.vr[i] = make_float4((float)s.v[0][i], (float)s.v[1][i], DIM == 3 ? (float)s.v[2][i] : 0.f,
                        (float)s.Pr[i]);
  s.rhof[i] = (float)s.rho[i];
}

// The operator bodies on a hit in FP32 (list entry = q | neighbour cell << 27;
// the separation is rebuilt from q's cell-relative position and the offset of
// its cell, exactly as the traversal computed it).
template <int DIM, int OP>
struct Proc32 {
  const State& s;
  const Consts& k;
  float4 pi4;
  float4 vp;   // own (vx, vy, vz, P/rho^2)
  float rhop;
  double acc, ax, ay, az, sx, sy, sz, wp, wg, ws;
  int c0, c1, c2;

  __device__ Proc32(const State& s_, const Consts& k_) : s(s_), k(k_) {
    acc = ax = ay = az = sx = sy = sz = wp = wg = ws = 0.0;
    vp = make_float4(0.f, 0.f, 0.f, 0.f);
    pi4 = vp;
    rhop = 0.f;
    c0 = c1 = c2 = 0;
  }

  __device__ __forceinline__ int entry(int q, int c, int tq) const {
    if (OP == SPH_OP_WALL_PRESSURE && tq != kFluid) return kCwSkip;
    return q | (c << kCwCellBits);
  }

  const float4* offs;  // the warp's neighbour-cell offsets (shared memory)

  __device__ __forceinline__ void process(const int* list, int stride, int cnt) {
    for (int t0 = 0; t0 < cnt; t0 += 32) {
      process_batch(list + (size_t)t0 * stride, stride, min(32, cnt - t0));
    }
  }

  // <= 32 hits summed in FP32, folded into the FP64 accumulators; the loads
  // of four hits are issued before their arithmetic
  __device__ __forceinline__ void process_batch(const int* list, int stride, int cnt) {
    float f0 = 0.f, f1 = 0.f, f2 = 0.f, f3 = 0.f, f4 = 0.f, f5 = 0.f;
    for (int t0 = 0; t0 < cnt; t0 += 4) {
      int e4[4];
      float4 p4[4], v4[4];
      float r4[4];
#pragma unroll
      for (int j = 0; j < 4; ++j)
        e4[j] = t0 + j < cnt ? __ldg(&list[(size_t)(t0 + j) * stride]) : kCwSkip;
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int q = e4[j] == kCwSkip ? 0 : e4[j] & kCwIndexMask;
        p4[j] = __ldg(&s.pl[q]);
        if (OP == SPH_OP_FORCE || OP == SPH_OP_WALL_PRESSURE) {
          v4[j] = __ldg(&s.vr[q]);
          r4[j] = __ldg(&s.rhof[q]);
        }
      }
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        if (t0 + j >= cnt) break;
        const int e = e4[j];
        if (e == kCwSkip) continue;  // a band candidate beyond the support
        const float4 off = offs[(unsigned)e >> kCwCellBits];
        const float4 pq = p4[j];
        const float hx = (pi4.x - pq.x) - off.x;
        const float hy = (pi4.y - pq.y) - off.y;
        const float hz = DIM == 3 ? (pi4.z - pq.z) - off.z : 0.f;
        float ss = hx * hx + hy * hy;
        if (DIM == 3) ss = ss + hz * hz;
        const float r = fsqrt(ss);
        const float kt = kt32(k, r);
        const bool fluid = __float_as_int(pq.w) == kFluid;
        if (OP != SPH_OP_FORCE || fluid) ++c0; else ++c1;
        if (OP == SPH_OP_DENSITY || OP == SPH_OP_DENSITY_REF) {
          // the shape t^4 (1 + 4x) only; m * C_w is applied in FP64 per batch
          const float t2 = kt * kt;
          f0 += (t2 * t2) * (5.f - 4.f * kt);
        } else if (OP == SPH_OP_WALL_PRESSURE) {
          const float w = kw32(k, r, kt);
          float gd = k.gf[0] * hx + k.gf[1] * hy;
          if (DIM == 3) gd += k.gf[2] * hz;
          const float rq = r4[j];
          const float Pq = v4[j].w * rq * rq;
          f0 += Pq * w;
          f1 += (rq * gd) * w;
          f2 += w;
        } else if (fluid) {
          const float4 vq = v4[j];
          const float rq = r4[j];
          const float ker = k.massf * krdw32(k, kt);
          const float dvx = vp.x - vq.x, dvy = vp.y - vq.y, dvz = vp.z - vq.z;
          float vdx = dvx * hx + dvy * hy;
          if (DIM == 3) vdx += dvz * hz;
          const float inv_rb = __fdividef(2.f, rhop + rq);
          float pi = 0.f;
          if (vdx < 0.f) {
            const float mu = __fdividef(k.h_smoothf * vdx, ss + k.eta2f);
            pi = (-k.alpha_c0f * mu) * inv_rb;
            ++c2;
          }
          const float cf = -ker * ((vp.w + vq.w) + pi);
          f0 += cf * hx;
          f1 += cf * hy;
          f2 += cf * hz;
          const float wx = k.massf * kw32(k, r, kt) * inv_rb;
          f3 -= wx * dvx;
          f4 -= wx * dvy;
          f5 -= wx * dvz;
        } else {
          const float cf = -(k.massf * krdw32(k, kt)) * (vp.w + v4[j].w);
          f0 += cf * hx;
          f1 += cf * hy;
          f2 += cf * hz;
        }
      }
    }
    if (OP == SPH_OP_DENSITY || OP == SPH_OP_DENSITY_REF) {
      acc += (k.mass * k.cw) * (double)f0;
    } else if (OP == SPH_OP_WALL_PRESSURE) {
      wp += (double)f0;
      wg += (double)f1;
      ws += (double)f2;
    } else {
      ax += (double)f0;
      ay += (double)f1;
      az += (double)f2;
      sx += (double)f3;
      sy += (double)f4;
      sz += (double)f5;
    }
  }
};

template <int DIM, int OP, int WARPS>
__global__ void __launch_bounds__(32 * WARPS) pair32_kernel(State s, Geometry g, Consts k,
                                                            BinScratch b, int self, int reset,
                                                            int fuse_eos, int list_mode) {
  __shared__ CwShared shared[WARPS];
  const int lane = threadIdx.x & 31;
  const int w = threadIdx.x >> 5;
  const int item = blockIdx.x * WARPS + w;
  int first = 0, count = 0;
  if (!cw_item(b, g, item, first, count)) return;  // warp-uniform
  const int i = first + lane;
  const bool valid = lane < count;
  const int ti = valid ? s.type[i] : -1;
  const int want = OP == SPH_OP_WALL_PRESSURE ? kWall : kFluid;
  CwTarget t;
  t.active = valid && ti == want;
  t.i = i;
  t.key = s.cell[first];
  decode_key(g, t.key, t.cx, t.cy, t.cz);
  t.pi4 = valid ? s.pl[i] : make_float4(0.f, 0.f, 0.f, 0.f);
  t.xp[0] = valid ? s.x[0][i] : 0.0;
  t.xp[1] = valid ? s.x[1][i] : 0.0;
  t.xp[2] = (DIM == 3 && valid) ? s.x[2][i] : 0.0;
  Proc32<DIM, OP> p(s, k);
  p.pi4 = t.pi4;
  p.offs = shared[w].offs;
  if (t.active) {
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
      p.vp = s.vr[i];
      p.rhop = s.rhof[i];
    }
  }
  cw_pass<DIM, OP>(s, g, k, b, shared[w], lane, item, t, p, list_mode);

  if (valid && !t.active) {
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
  } else if (t.active) {
    if (OP == SPH_OP_DENSITY || OP == SPH_OP_DENSITY_REF) {
      double acc = p.acc;
      if (self) acc = acc + k.mass * ker_w(k, 0.0);
      if (OP == SPH_OP_DENSITY) {
        s.rho[i] = acc;
        double Pr = s.Pr[i];
        if (fuse_eos) {
          const double ratio = acc / s.rho_ref[i];
          const double r2 = ratio * ratio;
          const double r4 = r2 * r2;
          const double r7 = (r4 * r2) * ratio;
          const double P = k.B * (r7 - 1.0);
          Pr = P / (acc * acc);
          s.P[i] = P;
          s.Pr[i] = Pr;
        }
        s.vr[i] = make_float4((float)s.v[0][i], (float)s.v[1][i],
                              DIM == 3 ? (float)s.v[2][i] : 0.f, (float)Pr);
        s.rhof[i] = (float)acc;
      } else {
        s.rho_ref[i] = acc;
      }
    } else if (OP == SPH_OP_WALL_PRESSURE) {
      const double P = p.ws > 0.0 ? (p.wp + p.wg) / p.ws : 0.0;
      const double Pr = P / (k.rho0 * k.rho0);
      s.P[i] = P;
      s.Pr[i] = Pr;
      s.rho[i] = k.rho0;
      s.vr[i] = make_float4((float)s.v[0][i], (float)s.v[1][i], DIM == 3 ? (float)s.v[2][i] : 0.f,
                            (float)Pr);
      s.rhof[i] = (float)k.rho0;
    } else {
      // the self term of the force adds exact zeros
      s.a[0][i] = p.ax;
      s.a[1][i] = p.ay;
      s.xs[0][i] = p.sx;
      s.xs[1][i] = p.sy;
      if (DIM == 3) {
        s.a[2][i] = p.az;
        s.xs[2][i] = p.sz;
      }
    }
  }
  cw_count<OP>(b, p.c0, p.c1, p.c2);
}

template <int DIM>
cudaError_t launch_dim(const LaunchCtx& c, const State& s, const Geometry& g, const Consts& k,
                       const BinScratch& b, int cap, int op, int self, int reset, int fuse_eos,
                       int aux_fresh, int list_mode) {
  const int W = k.warps;
  const int blocks = (b.max_items + W - 1) / W;
  if (!aux_fresh && (op == SPH_OP_FORCE || op == SPH_OP_WALL_PRESSURE)) {
    mark(c, SPH_KERNEL_UNARY, 0);
    aux_refresh_kernel<DIM><<<(cap + 255) / 256, 256, 0, c.stream>>>(s, b);
    mark(c, SPH_KERNEL_UNARY, 1);
  }
  const int kid = op == SPH_OP_FORCE           ? SPH_KERNEL_FORCE
                  : op == SPH_OP_WALL_PRESSURE ? SPH_KERNEL_WALL
                                               : SPH_KERNEL_DENSITY;
  mark(c, kid, 0);
  switch (op) {
    case SPH_OP_DENSITY:
      if (W == 2) pair32_kernel<DIM, SPH_OP_DENSITY, 2><<<blocks, 64, 0, c.stream>>>(s, g, k, b, self, reset, fuse_eos, 1);
      else if (W == 8) pair32_kernel<DIM, SPH_OP_DENSITY, 8><<<blocks, 256, 0, c.stream>>>(s, g, k, b, self, reset, fuse_eos, 1);
      else pair32_kernel<DIM, SPH_OP_DENSITY, 4><<<blocks, 128, 0, c.stream>>>(s, g, k, b, self, reset, fuse_eos, 1);
      break;
    case SPH_OP_DENSITY_REF:
      if (W == 2) pair32_kernel<DIM, SPH_OP_DENSITY_REF, 2><<<blocks, 64, 0, c.stream>>>(s, g, k, b, self, reset, 0, 1);
      else if (W == 8) pair32_kernel<DIM, SPH_OP_DENSITY_REF, 8><<<blocks, 256, 0, c.stream>>>(s, g, k, b, self, reset, 0, 1);
      else pair32_kernel<DIM, SPH_OP_DENSITY_REF, 4><<<blocks, 128, 0, c.stream>>>(s, g, k, b, self, reset, 0, 1);
      break;
    case SPH_OP_WALL_PRESSURE:
      if (W == 2) pair32_kernel<DIM, SPH_OP_WALL_PRESSURE, 2><<<blocks, 64, 0, c.stream>>>(s, g, k, b, 0, 0, 0, 0);
      else if (W == 8) pair32_kernel<DIM, SPH_OP_WALL_PRESSURE, 8><<<blocks, 256, 0, c.stream>>>(s, g, k, b, 0, 0, 0, 0);
      else pair32_kernel<DIM, SPH_OP_WALL_PRESSURE, 4><<<blocks, 128, 0, c.stream>>>(s, g, k, b, 0, 0, 0, 0);
      break;
    default:
      if (W == 2) pair32_kernel<DIM, SPH_OP_FORCE, 2><<<blocks, 64, 0, c.stream>>>(s, g, k, b, self, reset, 0, list_mode);
      else if (W == 8) pair32_kernel<DIM, SPH_OP_FORCE, 8><<<blocks, 256, 0, c.stream>>>(s, g, k, b, self, reset, 0, list_mode);
      else pair32_kernel<DIM, SPH_OP_FORCE, 4><<<blocks, 128, 0, c.stream>>>(s, g, k, b, self, reset, 0, list_mode);
      break;
  }
  mark(c, kid, 1);
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_pair_mixed(const LaunchCtx& c, const State& s, const Geometry& g,
                              const Consts& k, const BinScratch& b, int cap, int op, int self,
                              int reset, int fuse_eos, int aux_fresh, int lists_valid) {
  if (cap <= 0) return cudaSuccess;
  const int lm = lists_valid ? 2 : 0;
  return k.dim == 2 ? launch_dim<2>(c, s, g, k, b, cap, op, self, reset, fuse_eos, aux_fresh, lm)
                    : launch_dim<3>(c, s, g, k, b, cap, op, self, reset, fuse_eos, aux_fresh, lm);
}

}  // namespace sphgpu
