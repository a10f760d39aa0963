// sph_pair32.cu -- mixed-precision pair passes.
//
// Same traversal and the same candidate classification as the FP64 passes
// (FP32 test on cell-relative positions, FP64 band test with round-to-nearest
// intrinsics), so the set of pairs is identical to the FP64 path for the same
// positions.  What changes is the arithmetic on a hit:
//   * the separation is the FP32 cell-relative one computed by the scan
//     (x_p - x_q with both positions within one cell of the origin, so it is
//     accurate to ~2^-21 h), kept in the hit queue next to the index;
//   * kernel values, pressure, viscosity and XSPH terms are FP32, with the
//     neighbour's (v, P/rho^2, rho) read from a 20-byte FP32 copy;
//   * each queue batch (<= 16 hits) is summed in FP32 and folded into FP64
//     accumulators, so FP64 adds are per batch, not per hit;
//   * positions, the self term, the EOS, the wall-pressure quotient and the
//     time integration stay FP64.
// Built with FMA contraction (the FP64 band test uses explicit intrinsics).
#include "sph_launch.h"
#include "sphgpu.h"

namespace sphgpu {

namespace {

constexpr int kThreads32 = 128;
constexpr int kQ32 = 16;

__device__ __forceinline__ void warp_add(unsigned long long* dst, int v) {
  const int sum = __reduce_add_sync(0xffffffffu, v);
  if ((threadIdx.x & 31) == 0 && sum) atomicAdd(dst, (unsigned long long)sum);
}

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

template <int DIM, int OP>
__global__ void __launch_bounds__(kThreads32) pair32_kernel(State s, Geometry g, Consts k,
                                                            BinScratch b, int self, int reset,
                                                            int fuse_eos) {
  __shared__ float4 queue[kQ32][kThreads32];
  const int tid = threadIdx.x;
  const int n = *b.d_n;
  const int i = blockIdx.x * kThreads32 + tid;
  const int want = OP == SPH_OP_WALL_PRESSURE ? kWall : kFluid;
  int pairs = 0, c0 = 0, c1 = 0, c2 = 0;
  if (i < n && s.type[i] != want) {
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
    double acc = 0.0;
    double ax = 0.0, ay = 0.0, az = 0.0, sx = 0.0, sy = 0.0, sz = 0.0;
    double wp = 0.0, wg = 0.0, ws = 0.0;
    float4 vp = make_float4(0.f, 0.f, 0.f, 0.f);
    float rhop = 0.f;
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
      vp = s.vr[i];
      rhop = s.rhof[i];
    }

    int c = 0, j = 0, jend = 0;
    float ox = 0.f, oy = 0.f, oz = 0.f;
    bool more = true;
    while (more) {
      int cnt = 0;
      while (cnt < kQ32) {
        if (j >= jend) {
          if (c >= g.n_diff) { more = false; break; }
          const int nk = key + g.key_diff[c];
          ++c;
          if (nk < 1 || nk > g.key_max) continue;
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
        float dz = 0.f;
        float ss = dx * dx + dy * dy;
        if (DIM == 3) {
          dz = (pi4.z - pq.z) - oz;
          ss = ss + dz * dz;
        }
        if (ss > k.s_hi || q == i) continue;
        if (!(ss < k.s_lo) && !within_rn<DIM>(s, k, xp, q)) continue;
        ++pairs;
        const int tq = __float_as_int(pq.w);
        int e;
        if (OP == SPH_OP_WALL_PRESSURE) {
          if (tq != kFluid) continue;
          e = q;
        } else if (OP == SPH_OP_FORCE) {
          e = tq == kFluid ? q : -q - 1;
        } else {
          e = q;
        }
        queue[cnt++][tid] = make_float4(dx, dy, dz, __int_as_float(e));
      }
      // ---- process in FP32, fold the batch into FP64
      float f0 = 0.f, f1 = 0.f, f2 = 0.f, f3 = 0.f, f4 = 0.f, f5 = 0.f;
      for (int t = 0; t < cnt; ++t) {
        const float4 h = queue[t][tid];
        const int e = __float_as_int(h.w);
        float ss = h.x * h.x + h.y * h.y;
        if (DIM == 3) ss = ss + h.z * h.z;
        const float r = fsqrt(ss);
        const float kt = kt32(k, r);
        if (e >= 0) ++c0; else ++c1;
        if (OP == SPH_OP_DENSITY || OP == SPH_OP_DENSITY_REF) {
          // the shape t^4 (1 + 4x) only; m * C_w is applied in FP64 per batch
          const float t2 = kt * kt;
          f0 += (t2 * t2) * (5.f - 4.f * kt);
        } else if (OP == SPH_OP_WALL_PRESSURE) {
          const float w = kw32(k, r, kt);
          float gd = k.gf[0] * h.x + k.gf[1] * h.y;
          if (DIM == 3) gd += k.gf[2] * h.z;
          const float rq = __ldg(&s.rhof[e]);
          const float Pq = __ldg(&s.vr[e]).w * rq * rq;
          f0 += Pq * w;
          f1 += (rq * gd) * w;
          f2 += w;
        } else if (e >= 0) {
          const float4 vq = __ldg(&s.vr[e]);
          const float rq = __ldg(&s.rhof[e]);
          const float ker = k.massf * krdw32(k, kt);
          const float dvx = vp.x - vq.x, dvy = vp.y - vq.y, dvz = vp.z - vq.z;
          float vdx = dvx * h.x + dvy * h.y;
          if (DIM == 3) vdx += dvz * h.z;
          const float inv_rb = __fdividef(2.f, rhop + rq);
          float pi = 0.f;
          if (vdx < 0.f) {
            const float mu = __fdividef(k.h_smoothf * vdx, ss + k.eta2f);
            pi = (-k.alpha_c0f * mu) * inv_rb;
            ++c2;
          }
          const float cf = -ker * ((vp.w + vq.w) + pi);
          f0 += cf * h.x;
          f1 += cf * h.y;
          f2 += cf * h.z;
          const float wx = k.massf * kw32(k, r, kt) * inv_rb;
          f3 -= wx * dvx;
          f4 -= wx * dvy;
          f5 -= wx * dvz;
        } else {
          const float prq = __ldg(&s.vr[-e - 1]).w;
          const float cf = -(k.massf * krdw32(k, kt)) * (vp.w + prq);
          f0 += cf * h.x;
          f1 += cf * h.y;
          f2 += cf * h.z;
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
    if (OP == SPH_OP_DENSITY || OP == SPH_OP_DENSITY_REF) {
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
      const double P = ws > 0.0 ? (wp + wg) / ws : 0.0;
      const double Pr = P / (k.rho0 * k.rho0);
      s.P[i] = P;
      s.Pr[i] = Pr;
      s.rho[i] = k.rho0;
      s.vr[i] = make_float4((float)s.v[0][i], (float)s.v[1][i], DIM == 3 ? (float)s.v[2][i] : 0.f,
                            (float)Pr);
      s.rhof[i] = (float)k.rho0;
    } else {
      // the self term of the force adds exact zeros
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

template <int DIM>
cudaError_t launch_dim(const LaunchCtx& c, const State& s, const Geometry& g, const Consts& k,
                       const BinScratch& b, int cap, int op, int self, int reset, int fuse_eos,
                       int aux_fresh) {
  const int blocks = (cap + kThreads32 - 1) / kThreads32;
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
      pair32_kernel<DIM, SPH_OP_DENSITY><<<blocks, kThreads32, 0, c.stream>>>(s, g, k, b, self, reset, fuse_eos);
      break;
    case SPH_OP_DENSITY_REF:
      pair32_kernel<DIM, SPH_OP_DENSITY_REF><<<blocks, kThreads32, 0, c.stream>>>(s, g, k, b, self, reset, 0);
      break;
    case SPH_OP_WALL_PRESSURE:
      pair32_kernel<DIM, SPH_OP_WALL_PRESSURE><<<blocks, kThreads32, 0, c.stream>>>(s, g, k, b, 0, 0, 0);
      break;
    default:
      pair32_kernel<DIM, SPH_OP_FORCE><<<blocks, kThreads32, 0, c.stream>>>(s, g, k, b, self, reset, 0);
      break;
  }
  mark(c, kid, 1);
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_pair_mixed(const LaunchCtx& c, const State& s, const Geometry& g,
                              const Consts& k, const BinScratch& b, int cap, int op, int self,
                              int reset, int fuse_eos, int aux_fresh) {
  if (cap <= 0) return cudaSuccess;
  return k.dim == 2 ? launch_dim<2>(c, s, g, k, b, cap, op, self, reset, fuse_eos, aux_fresh)
                    : launch_dim<3>(c, s, g, k, b, cap, op, self, reset, fuse_eos, aux_fresh);
}

}  // namespace sphgpu
