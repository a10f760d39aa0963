// sph_pair32.cu -- mixed-precision pair passes.
//
// The candidate classification of the FP64 passes (FP32 test on
// cell-relative positions, FP64 band test with round-to-nearest intrinsics),
// so the set of pairs is the FP64 path's for the same positions.  The cells
// are the system's own (the reference's grid offset by 5/16 of a cell, the
// index from a product with 1/cell: the pair set does not depend on the
// grid).  What changes is the arithmetic on a hit:
//   * the separation is the FP32 cell-relative one (x_p - x_q with both
//     positions within one cell of their origins, accurate to ~2^-21 h);
//   * kernel values, pressure, viscosity and XSPH terms are FP32, with the
//     neighbour's (x, rho, v, P/rho^2) read from a 32-byte FP32 record;
//   * a lane's hits are summed in FP32 in batches of at most 32 and each
//     batch is folded into FP64 accumulators;
//   * positions, the self term, the EOS, the wall-pressure quotient and the
//     time integration stay FP64.
//
// Traversal (one warp per work item of <= 32 targets of one cell): every
// neighbour cell is visited in chunks of 32 candidates, staged into shared
// memory with coalesced loads.  The density and wall-pressure traversals
// test each staged candidate against the extent of the item's targets and
// take only the pairs of candidates one of which can be within reach (a
// chunk with none is skipped).  Per chunk each lane
//   A. classifies those candidates into a hit mask and a band mask (FP32
//      distances from broadcast reads); the density pass also evaluates the
//      kernel shape of every one of them here (zero beyond the support), so
//      all lanes do the same work,
//   B. resolves band candidates with the FP64 test, all lanes in lockstep,
//   C. (wall pressure, force) walks its hit mask in candidate order and
//      accumulates from shared memory, in the target's neighbour order.
// The density pass stores the final hit masks (4 bytes per lane per chunk,
// written coalesced) in slots counted during the binning; in the force pass
// of the same binning every lane walks its own stored masks, chunk by chunk,
// and loads each hit's record directly (no steps A and B).  An item whose
// slots do not fit the mask capacity traverses in both passes.
// Built with FMA contraction (the FP64 band test uses explicit intrinsics;
// any FP32 evaluation order stays within the classification band's margin).
#include <algorithm>

#include "sph_cellwarp.cuh"
#include "sph_launch.h"
#include "sphgpu.h"

namespace sphgpu {

namespace {

// Chunk table of the force pass's per-lane walk (3D items have ~54 chunks).
constexpr int kMaxChunks = 128;

// Candidates of a chunk are tested against the extent of the work item's
// active targets (the density and wall-pressure traversals; the force pass
// traverses only when its stored masks do not fit and tests every pair).
template <int OP>
constexpr bool kCull = OP != SPH_OP_FORCE;

template <int OP>
struct MxShared {
  static constexpr bool kRec = OP == SPH_OP_FORCE || OP == SPH_OP_WALL_PRESSURE;
  static constexpr int kTab = OP == SPH_OP_FORCE ? kMaxChunks : 1;
  // staged candidates of the force and wall-pressure traversals: the
  // 32-byte neighbour record (the density passes read the per-axis copies)
  float4 c0[kRec ? 32 : 1];    // (x, y, z) cell-relative, .w = signed rho
  float4 c1[kRec ? 32 : 1];    // (vx, vy, vz, P/rho^2)
  // the staged coordinates once more, one array per axis: step A reads two
  // candidates' coordinates as one 64-bit word for the packed FP32x2 tests
  alignas(16) float px[32];
  alignas(16) float py[32];
  alignas(16) float pz[32];
  unsigned fluid;              // wall pressure: bit u = candidate u is fluid
  float box[kCull<OP> ? 6 : 1];  // extent of the item's targets (low x, y, z; high x, y, z)
  float4 offs[27];             // offset of each neighbour cell from the target cell
  int cb[kTab];                // first candidate of each chunk of the item
  unsigned char cc[kTab];      // neighbour-cell number of each chunk
};

// coordinate of an empty staging slot: never within the support
constexpr float kFar = 1.0e18f;

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

// FP32 square root of a hit's squared distance (the hardware approximation;
// 0 for 0)
__device__ __forceinline__ float fsqrt(float ss) {
  float r;
  asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(ss));
  return r;
}

// The FP32 neighbour record of particle i: (cell-relative x, y, z, rho with
// the sign bit set for walls) and (vx, vy, vz, P/rho^2).
__device__ __forceinline__ void put_rec(const State& s, int i, const float4& pl, bool fluid,
                                        float rho, float vx, float vy, float vz, float pr) {
  const float rr = fabsf(rho);
  s.rec[2 * i] = make_float4(pl.x, pl.y, pl.z, fluid ? rr : -rr);
  s.rec[2 * i + 1] = make_float4(vx, vy, vz, pr);
}

// one 256-bit load of a record (32-byte aligned: the array is 256-byte
// aligned and records are 32 bytes)
__device__ __forceinline__ void ld_rec(const float4* p, float4& a, float4& b) {
  asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
      : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w)
      : "l"(p));
}

template <int DIM>
__global__ void __launch_bounds__(256) aux_refresh_kernel(State s, BinScratch b) {
  const int n = *b.d_n;
  const int i = blockIdx.x * 256 + threadIdx.x;
  if (i >= n) return;
  put_rec(s, i, s.pl[i], s.type[i] == kFluid, (float)s.rho[i], (float)s.v[0][i],
          (float)s.v[1][i], DIM == 3 ? (float)s.v[2][i] : 0.f, (float)s.Pr[i]);
}

// A lane's accumulators and the operator bodies on a hit, in FP32.
template <int DIM, int OP>
struct Acc32 {
  const Consts& k;
  float4 pi4;  // own cell-relative position
  float4 vp;   // own (vx, vy, vz, P/rho^2)
  float rhop;
  float f0, f1, f2, f3, f4, f5;  // the current FP32 batch
  int nh;                        // hits in the current batch
  double acc, ax, ay, az, sx, sy, sz, wp, wg, ws;
  int c0, c1, c2;

  __device__ explicit Acc32(const Consts& k_) : k(k_) {
    acc = ax = ay = az = sx = sy = sz = wp = wg = ws = 0.0;
    vp = make_float4(0.f, 0.f, 0.f, 0.f);
    pi4 = vp;
    rhop = 0.f;
    f0 = f1 = f2 = f3 = f4 = f5 = 0.f;
    nh = 0;
    c0 = c1 = c2 = 0;
  }

  // the batch into the FP64 accumulators
  __device__ __forceinline__ void fold() {
    if (nh == 0) return;
    if (OP == SPH_OP_DENSITY || OP == SPH_OP_DENSITY_REF) {
      acc += (k.mass * k.cw) * (double)f0;  // m * C_w applied in FP64
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
    f0 = f1 = f2 = f3 = f4 = f5 = 0.f;
    nh = 0;
  }

  // a hit on the neighbour with position / record (pq, vq) in a cell at
  // offset `off` from the target's cell
  __device__ __forceinline__ void hit(const float4& pq, const float4& vq, const float4& off) {
    hit_rel(pq, vq, pi4.x - off.x, pi4.y - off.y, pi4.z - off.z);
  }
  // the same with the target's position relative to the neighbour's cell
  // (ax, ay, az) at hand, as step A forms the separations
  __device__ __forceinline__ void hit_rel(const float4& pq, const float4& vq, float ax, float ay,
                                          float az) {
    const float hx = ax - pq.x;
    const float hy = ay - pq.y;
    const float hz = DIM == 3 ? az - pq.z : 0.f;
    float ss = hx * hx + hy * hy;
    if (DIM == 3) ss = ss + hz * hz;
    const float r = fsqrt(ss);
    const float kt = kt32(k, r);
    // the density and wall-pressure passes count their hits per chunk
    if (OP == SPH_OP_FORCE) ++nh;
    if (OP == SPH_OP_DENSITY || OP == SPH_OP_DENSITY_REF) {
      // the shape t^4 (1 + 4x) only; m * C_w is applied per batch
      const float t2 = kt * kt;
      f0 += (t2 * t2) * (5.f - 4.f * kt);
    } else if (OP == SPH_OP_WALL_PRESSURE) {
      // Adami, Hu & Adams (2012) wall pressure, g . (x_w - x_f)
      const float w = kw32(k, r, kt);
      float gd = k.gf[0] * hx + k.gf[1] * hy;
      if (DIM == 3) gd += k.gf[2] * hz;
      const float rq = fabsf(pq.w);
      // P from the record's pressure term (P/rho^2, or P/rho0^2 under the
      // linear EOS)
      const float Pq = k.eos == 1 ? vq.w * (k.rho0f * k.rho0f) : vq.w * rq * rq;
      f0 += Pq * w;
      f1 += (rq * gd) * w;
      f2 += w;
    } else if (!signbit(pq.w)) {
      ++c0;
      // pressure (collapse_symplectic.jl:114-118) + Monaghan viscosity + XSPH
      const float rq = pq.w;
      const float ker = k.massf * krdw32(k, kt);
      const float dvx = vp.x - vq.x, dvy = vp.y - vq.y, dvz = vp.z - vq.z;
      float vdx = dvx * hx + dvy * hy;
      if (DIM == 3) vdx += dvz * hz;
      const float inv_rb = __fdividef(2.f, rhop + rq);
      // Monaghan viscosity only for approaching pairs (v.x < 0); evaluated
      // without a branch: mu = 0 otherwise
      const float mu = __fdividef(k.h_smoothf * fminf(vdx, 0.f), ss + k.eta2f);
      const float pi = (-k.alpha_c0f * mu) * inv_rb;
      c2 += vdx < 0.f ? 1 : 0;
      const float cf = -ker * ((vp.w + vq.w) + pi);
      f0 += cf * hx;
      f1 += cf * hy;
      f2 += cf * hz;
      const float wx = k.massf * kw32(k, r, kt) * inv_rb;
      f3 -= wx * dvx;
      f4 -= wx * dvy;
      f5 -= wx * dvz;
    } else {
      ++c1;
      // wall neighbour: pressure term with the wall pressure
      const float cf = -(k.massf * krdw32(k, kt)) * (vp.w + vq.w);
      f0 += cf * hx;
      f1 += cf * hy;
      f2 += cf * hz;
    }
  }
};

// The extent of the item's active targets (cell-relative FP32 positions) into
// sh.box; the caller syncs the warp before it is read.
template <int OP>
__device__ __forceinline__ void mx_item_box(MxShared<OP>& sh, int lane, const CwTarget& t) {
  float lx = t.active ? t.pi4.x : kFar, ly = t.active ? t.pi4.y : kFar;
  float lz = t.active ? t.pi4.z : kFar;
  float hx = t.active ? t.pi4.x : -kFar, hy = t.active ? t.pi4.y : -kFar;
  float hz = t.active ? t.pi4.z : -kFar;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    lx = fminf(lx, __shfl_xor_sync(0xffffffffu, lx, o));
    ly = fminf(ly, __shfl_xor_sync(0xffffffffu, ly, o));
    lz = fminf(lz, __shfl_xor_sync(0xffffffffu, lz, o));
    hx = fmaxf(hx, __shfl_xor_sync(0xffffffffu, hx, o));
    hy = fmaxf(hy, __shfl_xor_sync(0xffffffffu, hy, o));
    hz = fmaxf(hz, __shfl_xor_sync(0xffffffffu, hz, o));
  }
  if (lane == 0) {
    sh.box[0] = lx; sh.box[1] = ly; sh.box[2] = lz;
    sh.box[3] = hx; sh.box[4] = hy; sh.box[5] = hz;
  }
}

// Whether candidate c of a neighbour cell at offset `off` can be within the
// support of any target of the item.  The box is taken into the neighbour
// cell's frame as the targets' own positions are (a - off for every target
// coordinate a), so it holds every target's (ax, ay, az); the squared gap
// between c and the box is formed with the operations (and so the rounding)
// of step A's squared distance.  Rounding is monotone, so the gap along every
// axis is at most |ax - c.x| for every target and the squared gap at most
// every target's FP32 squared distance: a candidate beyond s_hi here is
// beyond it for every target.
template <int DIM, int OP>
__device__ __forceinline__ bool mx_near_box(const MxShared<OP>& sh, const float4& off,
                                            const float4& c, float s_hi) {
  const float gx = fmaxf(fmaxf(__fsub_rn(__fsub_rn(sh.box[0], off.x), c.x),
                               __fsub_rn(c.x, __fsub_rn(sh.box[3], off.x))), 0.f);
  const float gy = fmaxf(fmaxf(__fsub_rn(__fsub_rn(sh.box[1], off.y), c.y),
                               __fsub_rn(c.y, __fsub_rn(sh.box[4], off.y))), 0.f);
  float g2 = __fmaf_rn(gy, gy, __fmul_rn(gx, gx));
  if (DIM == 3) {
    const float gz = fmaxf(fmaxf(__fsub_rn(__fsub_rn(sh.box[2], off.z), c.z),
                                 __fsub_rn(c.z, __fsub_rn(sh.box[5], off.z))), 0.f);
    g2 = __fmaf_rn(gz, gz, g2);
  }
  return g2 <= s_hi;
}

// Stages candidates [base, base + m) of one neighbour cell; empty slots get a
// far-away position and the type of no operator's neighbour.  CLASSIFY: the
// chunk goes through step A, which also wants the per-axis copies; the
// return value is then the chunk's live pairs: bit 2j set when candidate 2j
// or 2j + 1 is near the item's box (and, for the wall pressure, fluid), every
// pair for the force pass.  `off`: the neighbour cell's offset.
template <int DIM, int OP, bool CLASSIFY>
__device__ __forceinline__ unsigned mx_stage(const State& s, const Consts& k, MxShared<OP>& sh,
                                             int lane, int base, int m, const float4& off) {
  __syncwarp();
  float4 c;
  if (MxShared<OP>::kRec) {
    if (lane < m) {
      float4 v;
      ld_rec(s.rec + 2 * (base + lane), c, v);
      sh.c0[lane] = c;
      sh.c1[lane] = v;
    } else {
      c = make_float4(kFar, kFar, kFar, -1.f);
      sh.c0[lane] = c;
    }
  } else {
    c = lane < m ? __ldg(&s.pl[base + lane]) : make_float4(kFar, kFar, kFar, __int_as_float(-1));
  }
  unsigned live = 0u;
  if (CLASSIFY) {
    sh.px[lane] = c.x;
    sh.py[lane] = c.y;
    sh.pz[lane] = c.z;
    if (OP == SPH_OP_WALL_PRESSURE) {
      const unsigned f = __ballot_sync(0xffffffffu, !signbit(c.w));
      if (lane == 0) sh.fluid = f;
    }
    if (kCull<OP>) {
      bool near = mx_near_box<DIM>(sh, off, c, k.s_hi);
      if (OP == SPH_OP_WALL_PRESSURE) near = near && !signbit(c.w);
      live = __ballot_sync(0xffffffffu, near);
      live = (live | (live >> 1)) & 0x55555555u;
    } else {
      live = 0x55555555u;
    }
  }
  __syncwarp();
  return live;
}

// FP32 square root (the hardware approximation; a subnormal or zero square
// gives 0).
__device__ __forceinline__ float sqrt_approx(float x) {
  float r;
  asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// Step A over the live pairs `pl` of the 32 staged candidates (bit 2j: the
// pair 2j, 2j + 1), for a target at (ax, ay, az) relative to their cell:
// the hit mask (inside or in the band) and the band mask.  Candidates of the
// other pairs are beyond the support of every target of the item.  The
// sixteen pairs are unrolled from pair 15 down; the skip of a pair is the
// same for the whole warp.  Two candidates per packed FP32x2 operation; the
// decisions are the signs of ss - s_hi' (s_hi' the float after s_hi; set:
// ss <= s_hi) and ss - s_lo (set: below the band), exact in FP32,
// funnel-shifted into the masks (a skipped pair shifts in zeros).  DENS: also
// the density's kernel shape t^4 (5 - 4t), t = 1 - min(r, h)/h, of every
// candidate of the live pairs, summed into two FP32 partial sums; beyond the
// support it is zero up to the rounding of r (|t| < 2^-23), and SELF zeroes
// the target's own candidate (self_u).
template <int DIM, int OP, bool DENS, bool SELF>
__device__ __forceinline__ void mx_step_a(const MxShared<OP>& sh, const Consts& k, float ax,
                                          float ay, float az, unsigned pl, int self_u,
                                          unsigned& hit, unsigned& band, float& fc) {
  const unsigned long long cx = f2_pack(ax, ax), cy = f2_pack(ay, ay), cz = f2_pack(az, az);
  const float shi1 = __int_as_float(__float_as_int(k.s_hi) + 1);
  const unsigned long long shi = f2_pack(shi1, shi1), slo = f2_pack(k.s_lo, k.s_lo);
  const unsigned long long* x2 = reinterpret_cast<const unsigned long long*>(sh.px);
  const unsigned long long* y2 = reinterpret_cast<const unsigned long long*>(sh.py);
  const unsigned long long* z2 = reinterpret_cast<const unsigned long long*>(sh.pz);
  const unsigned long long minvh = f2_pack(-k.inv_hf, -k.inv_hf);
  const unsigned long long one = f2_pack(1.f, 1.f), five = f2_pack(5.f, 5.f);
  const unsigned long long m4 = f2_pack(-4.f, -4.f);
  const unsigned long long keep = (self_u & 1) ? 0x00000000ffffffffull : 0xffffffff00000000ull;
  unsigned long long acc = 0ull;
  unsigned in = 0u, low = 0u;  // bit u: candidate u within s_hi / below the band
#pragma unroll
  for (int i2 = 15; i2 >= 0; --i2) {
    if (pl & (1u << (2 * i2))) {
      const unsigned long long dx = f2_sub(cx, x2[i2]);
      const unsigned long long dy = f2_sub(cy, y2[i2]);
      unsigned long long ss = f2_fma(dy, dy, f2_mul(dx, dx));
      if (DIM == 3) {
        const unsigned long long dz = f2_sub(cz, z2[i2]);
        ss = f2_fma(dz, dz, ss);
      }
      const unsigned long long dh = f2_sub(ss, shi);
      const unsigned long long dl = f2_sub(ss, slo);
      in = __funnelshift_l((unsigned)(dh >> 32), in, 1);
      in = __funnelshift_l((unsigned)dh, in, 1);
      low = __funnelshift_l((unsigned)(dl >> 32), low, 1);
      low = __funnelshift_l((unsigned)dl, low, 1);
      if (DENS) {
        const float r1 = fminf(sqrt_approx(__uint_as_float((unsigned)ss)), k.hf);
        const float r2 = fminf(sqrt_approx(__uint_as_float((unsigned)(ss >> 32))), k.hf);
        const unsigned long long t = f2_fma(f2_pack(r1, r2), minvh, one);  // 1 - r/h
        const unsigned long long t2 = f2_mul(t, t);
        unsigned long long w = f2_mul(f2_mul(t2, t2), f2_fma(m4, t, five));
        if (SELF && (self_u >> 1) == i2) w &= keep;
        acc = f2_add(acc, w);
      }
    } else {
      in <<= 2;
      low <<= 2;
    }
  }
  unsigned h = in;
  if (OP == SPH_OP_WALL_PRESSURE) h &= sh.fluid;
  hit = h;
  band = ~low & h;
  if (DENS) fc = __uint_as_float((unsigned)acc) + __uint_as_float((unsigned)(acc >> 32));
}

// Step B: the reference's FP64 test for every band candidate, the lanes
// taking their band candidates together (on the benchmark lattices many
// candidates lie exactly at r = h).
template <int DIM>
__device__ __forceinline__ void mx_resolve(const State& s, const Consts& k, const CwTarget& t,
                                           int base, unsigned& hit, unsigned band) {
  while (__any_sync(0xffffffffu, band != 0u)) {
    if (band) {
      const int u = __ffs(band) - 1;
      band &= band - 1u;
      if (!within_rn<DIM>(s, k, t.xp, base + u)) hit &= ~(1u << u);
    }
  }
}

// Force pass over stored masks: the chunk table of the item (first candidate
// and neighbour-cell number of every chunk, in traversal order).  False when
// it does not match the slots the binning counted or does not fit.
__device__ __forceinline__ bool mx_chunk_table(const Geometry& g, const BinScratch& b,
                                               MxShared<SPH_OP_FORCE>& sh, int lane,
                                               const CwTarget& t, int nc) {
  int st = 0, nch = 0;
  if (lane < g.n_diff) {
    const int nk = t.key + g.key_diff[lane];
    if (nk >= 1 && nk <= g.key_max) {
      st = __ldg(&b.cell_start[nk]);
      nch = (__ldg(&b.cell_start[nk + 1]) - st + 31) >> 5;
    }
  }
  int incl = nch;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int v = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += v;
  }
  const int total = __shfl_sync(0xffffffffu, incl, 31);
  if (total != nc || total > kMaxChunks) return false;
  for (int j = 0, f = incl - nch; j < nch; ++j, ++f) {
    sh.cb[f] = st + 32 * j;
    sh.cc[f] = (unsigned char)lane;
  }
  __syncwarp();
  return true;
}

// Force pass over stored masks: every lane walks its own hits (chunk by
// chunk, bit by bit: the traversal order) and loads each neighbour's record
// directly, so lanes never wait for one another within a chunk.  Two hits per
// step keep two record loads in flight.
struct MxCursor {
  int gi;       // current chunk
  unsigned cm;  // its bits not yet taken
  unsigned nm;  // mask of chunk gi + step (loaded ahead)
  int step;     // the warps sharing the item: this warp takes every step-th chunk
};

__device__ __forceinline__ int mx_next(const unsigned* mrow, const MxShared<SPH_OP_FORCE>& sh,
                                       int nc, MxCursor& c, int& cell) {
  while (c.cm == 0u && c.gi + c.step < nc) {
    c.gi += c.step;
    c.cm = c.nm;
    if (c.gi + c.step < nc) c.nm = __ldg(mrow + (size_t)(c.gi + c.step) * 32);
  }
  if (c.cm == 0u) return -1;
  const int u = __ffs(c.cm) - 1;
  c.cm &= c.cm - 1u;
  cell = sh.cc[c.gi];
  return sh.cb[c.gi] + u;
}

template <int DIM>
__device__ __forceinline__ void mx_walk(const State& s, const BinScratch& b,
                                        const MxShared<SPH_OP_FORCE>& sh, int lane,
                                        const CwTarget& t, Acc32<DIM, SPH_OP_FORCE>& a, int ck,
                                        int nc, int part, int split) {
  const unsigned* mrow = b.ck_mask + (size_t)ck * 32 + lane;
  MxCursor cur;
  cur.step = split;
  cur.gi = t.active ? part - split : nc;
  cur.cm = 0u;
  cur.nm = t.active && part < nc ? __ldg(mrow + (size_t)part * 32) : 0u;
  int qa = -1, qb = -1, ca = 0, cb = 0;
  for (;;) {
    // take two hits per step until every lane is done or a lane with hits
    // left would overflow its FP32 batch; then fold every lane's batch
    unsigned w;
    for (;;) {
      if (qa < 0) qa = mx_next(mrow, sh, nc, cur, ca);
      if (qb < 0) qb = mx_next(mrow, sh, nc, cur, cb);
      const bool work = qa >= 0;
      const bool full = a.nh > 30;
      w = __reduce_or_sync(0xffffffffu, (work ? 1u : 0u) | ((work && full) ? 2u : 0u));
      if (w != 1u) break;
      if (work) {
        float4 pa, va, pb, vb;
        ld_rec(s.rec + 2 * qa, pa, va);
        if (qb >= 0) ld_rec(s.rec + 2 * qb, pb, vb);
        a.hit(pa, va, sh.offs[ca]);
        if (qb >= 0) a.hit(pb, vb, sh.offs[cb]);
        qa = qb = -1;
      }
    }
    if (w == 0u) return;
    a.fold();
  }
}

// The traversal of one item's neighbour cells, chunk by chunk (steps A-C);
// `read`: masks stored by the density pass are used where they exist.
template <int DIM, int OP>
__device__ __forceinline__ void mx_traverse(const State& s, const Geometry& g, const Consts& k,
                                            const BinScratch& b, MxShared<OP>& sh, int lane,
                                            const CwTarget& t, Acc32<DIM, OP>& a, int ck, int nc,
                                            bool read, bool store, int part, int split) {
  constexpr bool kDens = OP == SPH_OP_DENSITY || OP == SPH_OP_DENSITY_REF;
  if (kCull<OP>) {
    mx_item_box(sh, lane, t);
    __syncwarp();
  }
  int gi = 0;         // chunk number in the item's neighbour sequence
  int mine = part;    // the next chunk this warp takes
  for (int c = 0; c < g.n_diff; ++c) {
    const int nk = t.key + g.key_diff[c];
    if (nk < 1 || nk > g.key_max) continue;  // core.jl:98
    if (OP == SPH_OP_WALL_PRESSURE && __ldg(&b.cell_fluid[nk]) == 0) continue;
    const int st = __ldg(&b.cell_start[nk]);
    const int en = __ldg(&b.cell_start[nk + 1]);
    const float4 off = sh.offs[c];
    const float ax = t.pi4.x - off.x, ay = t.pi4.y - off.y, az = t.pi4.z - off.z;
    for (int base = st; base < en; base += 32) {
      const int m = min(32, en - base);
      if (split > 1) {
        if (gi != mine) {  // another warp's chunk
          ++gi;
          continue;
        }
        mine += split;
      }
      unsigned mask;
      float fc = 0.f;  // density: the chunk's FP32 shape sum
      if (read && gi < nc) {
        mask = t.active ? __ldg(&b.ck_mask[((size_t)ck + gi) * 32 + lane]) : 0u;
        ++gi;
        if (!__any_sync(0xffffffffu, mask != 0u)) continue;
        mx_stage<DIM, OP, false>(s, k, sh, lane, base, m, off);
      } else {
        const unsigned pl = mx_stage<DIM, OP, true>(s, k, sh, lane, base, m, off);
        if (pl == 0u) {
          // no candidate of the chunk is within reach of the item's box
          if (store && gi < nc) b.ck_mask[((size_t)ck + gi) * 32 + lane] = 0u;
          ++gi;
          continue;
        }
        unsigned band;
        const int self_u = t.i - base;  // core.jl:105: p == q is skipped
        if (__any_sync(0xffffffffu, self_u >= 0 && self_u < 32))
          mx_step_a<DIM, OP, kDens, true>(sh, k, ax, ay, az, pl, self_u, mask, band, fc);
        else
          mx_step_a<DIM, OP, kDens, false>(sh, k, ax, ay, az, pl, self_u, mask, band, fc);
        if (self_u >= 0 && self_u < 32) {
          mask &= ~(1u << self_u);
          band &= ~(1u << self_u);
        }
        if (!t.active) mask = band = 0u;
        if (__any_sync(0xffffffffu, band != 0u)) mx_resolve<DIM>(s, k, t, base, mask, band);
        if (store && gi < nc) b.ck_mask[((size_t)ck + gi) * 32 + lane] = mask;
        ++gi;
      }
      // keep every lane's FP32 batch at <= 32 hits (one decision per warp)
      if (__any_sync(0xffffffffu, a.nh + __popc(mask) > 32)) a.fold();
      if (OP != SPH_OP_FORCE) {
        const int hits = __popc(mask);
        a.nh += hits;
        a.c0 += hits;
      }
      if constexpr (kDens) {
        // the shapes step A summed (a band candidate the FP64 test rejects
        // lies at r = h within 2^-14 h: its shape is below 1e-16, as are
        // the others' beyond the support)
        a.f0 += fc;
      } else {
        while (mask) {
          const int u = __ffs(mask) - 1;
          mask &= mask - 1u;
          float4 vq = make_float4(0.f, 0.f, 0.f, 0.f);
          if constexpr (MxShared<OP>::kRec) vq = sh.c1[u];
          a.hit_rel(sh.c0[u], vq, ax, ay, az);
        }
      }
    }
  }
  a.fold();
}

// list_mode: 0 traverse; 1 traverse and store the hit masks (density
// passes); 2 read the masks stored by the density pass of this binning.
// The item's chunks are shared by `split` warps: this one takes the chunks
// gi with gi % split == part.
template <int DIM, int OP>
__device__ __forceinline__ void mx_pass(const State& s, const Geometry& g, const Consts& k,
                                        const BinScratch& b, MxShared<OP>& sh, int lane, int item,
                                        const CwTarget& t, Acc32<DIM, OP>& a, int list_mode,
                                        int part, int split) {
  // this item's mask slots: the binning counted every cell's chunks
  int ck = -1, nc = 0;
  if (list_mode != 0 && b.ck_mask) {
    const int i0 = __ldg(&b.item_off[t.key]);
    const int ni = __ldg(&b.item_off[t.key + 1]) - i0;
    const int co = __ldg(&b.chunk_off[t.key]);
    nc = ni > 0 ? (__ldg(&b.chunk_off[t.key + 1]) - co) / ni : 0;
    const long long start = (long long)co + (long long)(item - i0) * nc;
    if (start + nc <= (long long)b.ck_cap) ck = (int)start;
  }
  // slots beyond the counted nc (types changed since the binning) are
  // neither read nor written
  const bool read = OP == SPH_OP_FORCE && list_mode == 2 && ck >= 0;
  const bool store = list_mode == 1 && ck >= 0;
  if (lane < g.n_diff) {
    const int nk = t.key + g.key_diff[lane];
    sh.offs[lane] = (nk >= 1 && nk <= g.key_max) ? cw_offset(g, k, t, nk)
                                                 : make_float4(0.f, 0.f, 0.f, 0.f);
  }
  __syncwarp();
  if constexpr (OP == SPH_OP_FORCE) {
    if (read && mx_chunk_table(g, b, sh, lane, t, nc)) {
      mx_walk<DIM>(s, b, sh, lane, t, a, ck, nc, part, split);
      a.fold();
      return;
    }
  }
  mx_traverse<DIM, OP>(s, g, k, b, sh, lane, t, a, ck, nc, read, store, part, split);
}

// The FP64 accumulators a warp of a shared item hands to the item's first
// warp (by lane): density 1, wall pressure 3, force 6, written over the
// warp's own staging area once its traversal is done.
template <int OP>
constexpr int kCombWords = (OP == SPH_OP_DENSITY || OP == SPH_OP_DENSITY_REF) ? 1
                           : OP == SPH_OP_WALL_PRESSURE                       ? 3
                                                                              : 6;

template <int OP>
__device__ __forceinline__ double (*comb_of(MxShared<OP>& sh))[32] {
  static_assert(sizeof(MxShared<OP>) >= sizeof(double) * 32 * kCombWords<OP>,
                "a warp's staging area holds its partial sums");
  return reinterpret_cast<double (*)[32]>(&sh);
}

template <int DIM, int OP>
__device__ __forceinline__ void comb_put(double (*c)[32], int lane, const Acc32<DIM, OP>& p) {
  // every lane of the warp has left the staging area (the caller syncs)
  if (OP == SPH_OP_DENSITY || OP == SPH_OP_DENSITY_REF) {
    c[0][lane] = p.acc;
  } else if (OP == SPH_OP_WALL_PRESSURE) {
    c[0][lane] = p.wp;
    c[1][lane] = p.wg;
    c[2][lane] = p.ws;
  } else {
    c[0][lane] = p.ax;
    c[1][lane] = p.ay;
    c[2][lane] = p.az;
    c[3][lane] = p.sx;
    c[4][lane] = p.sy;
    c[5][lane] = p.sz;
  }
}

template <int DIM, int OP>
__device__ __forceinline__ void comb_add(const double (*c)[32], int lane, Acc32<DIM, OP>& p) {
  if (OP == SPH_OP_DENSITY || OP == SPH_OP_DENSITY_REF) {
    p.acc += c[0][lane];
  } else if (OP == SPH_OP_WALL_PRESSURE) {
    p.wp += c[0][lane];
    p.wg += c[1][lane];
    p.ws += c[2][lane];
  } else {
    p.ax += c[0][lane];
    p.ay += c[1][lane];
    p.az += c[2][lane];
    p.sx += c[3][lane];
    p.sy += c[4][lane];
    p.sz += c[5][lane];
  }
}

// One work item (<= 32 targets of one cell) per `split` warps of the block
// (k.split: 1, 2 or 4, dividing WARPS): warp `part` of an item takes every
// split-th chunk of the neighbour sequence, and the item's first warp adds
// the others' FP64 sums to its own in warp order before the epilogue.
// SPLIT = false compiles the one-warp-per-item code alone (its registers).
template <int DIM, int OP, int WARPS, bool SPLIT>
__device__ __forceinline__ void pair32_body(const State& s, const Geometry& g, const Consts& k,
                                            const BinScratch& b, int self, int reset,
                                            int fuse_eos, int list_mode, int blk,
                                            MxShared<OP>* shared) {
  const int lane = threadIdx.x & 31;
  const int w = threadIdx.x >> 5;
  const int split = SPLIT ? k.split : 1;  // block-uniform: 1, 2 or 4
  const int lg = split >> 1;  // log2(split)
  const int item = (blk * WARPS + w) >> lg;
  const int part = w & (split - 1);
  int first = 0, count = 0;
  const bool has = cw_item(b, g, item, first, count);  // warp-uniform
  if (split == 1 && !has) return;  // no barriers below when the item is one warp's
  const int i = first + lane;
  const bool valid = has && lane < count;
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
  Acc32<DIM, OP> p(k);
  p.pi4 = t.pi4;
  if (t.active && part == 0) {
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
    }
  }
  if (OP == SPH_OP_FORCE && t.active) {
    float4 r0;
    ld_rec(s.rec + 2 * i, r0, p.vp);
    p.rhop = fabsf(r0.w);
  }
  if (__any_sync(0xffffffffu, t.active))
    mx_pass<DIM, OP>(s, g, k, b, shared[w], lane, item, t, p, list_mode, part, split);
  if (split > 1) {
    // the other warps' sums to the item's first warp, added in warp order
    __syncwarp();
    if (part > 0) comb_put<DIM, OP>(comb_of(shared[w]), lane, p);
    __syncthreads();
    if (part == 0)
      for (int o = 1; o < split; ++o) comb_add<DIM, OP>(comb_of(shared[w + o]), lane, p);
    cw_count<OP>(b, p.c0, p.c1, p.c2);
    if (part > 0 || !has) return;
  }
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
          double P;
          eos_eval(k, acc, s.rho_ref[i], P, Pr);
          s.P[i] = P;
          s.Pr[i] = Pr;
        }
        put_rec(s, i, t.pi4, true, (float)acc, (float)s.v[0][i], (float)s.v[1][i],
                DIM == 3 ? (float)s.v[2][i] : 0.f, (float)Pr);
      } else {
        s.rho_ref[i] = acc;
      }
    } else if (OP == SPH_OP_WALL_PRESSURE) {
      const double P = p.ws > 0.0 ? (p.wp + p.wg) / p.ws : 0.0;
      const double Pr = P / (k.rho0 * k.rho0);
      s.P[i] = P;
      s.Pr[i] = Pr;
      s.rho[i] = k.rho0;
      put_rec(s, i, t.pi4, false, (float)k.rho0, (float)s.v[0][i], (float)s.v[1][i],
              DIM == 3 ? (float)s.v[2][i] : 0.f, (float)Pr);
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
  if (split == 1) cw_count<OP>(b, p.c0, p.c1, p.c2);
}

// The force pass (latency bound on its record gathers) runs at
// SPH_FORCE_BLOCKS blocks of 4 warps per SM (8: 64 registers); 0 leaves the
// other passes to the compiler.
#ifndef SPH_FORCE_BLOCKS
#define SPH_FORCE_BLOCKS 8
#endif
template <int OP, int WARPS>
constexpr int kMinBlocks32 = (OP == SPH_OP_FORCE && WARPS == 4) ? SPH_FORCE_BLOCKS : 0;

template <int DIM, int OP, int WARPS, bool SPLIT>
__global__ void __launch_bounds__(32 * WARPS, kMinBlocks32<OP, WARPS>) pair32_kernel(State s, Geometry g, Consts k,
                                                            BinScratch b, int self, int reset,
                                                            int fuse_eos, int list_mode) {
  __shared__ MxShared<OP> shared[WARPS];
  pair32_body<DIM, OP, WARPS, SPLIT>(s, g, k, b, self, reset, fuse_eos, list_mode, blockIdx.x,
                                     shared);
}

// fused batches: block i works on map[i] = (member, block of that member)
template <int DIM, int OP, int WARPS, bool SPLIT>
__global__ void __launch_bounds__(32 * WARPS) pair32_fused_kernel(
    const MemberArgs* __restrict__ margs, const int2* __restrict__ map, int self, int reset,
    int fuse_eos, int list_mode) {
  __shared__ MxShared<OP> shared[WARPS];
  const int2 e = map[blockIdx.x];
  const MemberArgs& m = margs[e.x];
  pair32_body<DIM, OP, WARPS, SPLIT>(m.cur, m.g, m.k, m.b, self, reset, fuse_eos, list_mode, e.y,
                                     shared);
}

template <int DIM, int OP, int WARPS>
void fused_launch(const FusedBatch& fb, int p, cudaStream_t st, int self, int reset, int fuse_eos,
                  int list_mode) {
  if (fb.split)
    pair32_fused_kernel<DIM, OP, WARPS, true><<<(unsigned)fb.blocks[kShapeItems], 32 * WARPS, 0, st>>>(
        fb.args[p], fb.map[kShapeItems], self, reset, fuse_eos, list_mode);
  else
    pair32_fused_kernel<DIM, OP, WARPS, false><<<(unsigned)fb.blocks[kShapeItems], 32 * WARPS, 0, st>>>(
        fb.args[p], fb.map[kShapeItems], self, reset, fuse_eos, list_mode);
}

template <int DIM, int OP>
void fused_launch_w(const FusedBatch& fb, int p, cudaStream_t st, int self, int reset,
                    int fuse_eos, int list_mode) {
  if (fb.warps == 2)
    fused_launch<DIM, OP, 2>(fb, p, st, self, reset, fuse_eos, list_mode);
  else if (fb.warps == 8)
    fused_launch<DIM, OP, 8>(fb, p, st, self, reset, fuse_eos, list_mode);
  else
    fused_launch<DIM, OP, 4>(fb, p, st, self, reset, fuse_eos, list_mode);
}

template <int DIM>
cudaError_t launch_fused_dim(const LaunchCtx& c, const FusedBatch& fb, int p, int op, int self,
                             int reset, int fuse_eos, int list_mode) {
  const int kid = op == SPH_OP_FORCE           ? SPH_KERNEL_FORCE
                  : op == SPH_OP_WALL_PRESSURE ? SPH_KERNEL_WALL
                                               : SPH_KERNEL_DENSITY;
  mark(c, kid, 0);
  switch (op) {
    case SPH_OP_DENSITY:
      fused_launch_w<DIM, SPH_OP_DENSITY>(fb, p, c.stream, self, reset, fuse_eos, 1);
      break;
    case SPH_OP_WALL_PRESSURE:
      fused_launch_w<DIM, SPH_OP_WALL_PRESSURE>(fb, p, c.stream, 0, 0, 0, 0);
      break;
    case SPH_OP_FORCE:
      fused_launch_w<DIM, SPH_OP_FORCE>(fb, p, c.stream, self, reset, 0, list_mode);
      break;
    default:
      return cudaErrorNotSupported;
  }
  mark(c, kid, 1);
  return cudaGetLastError();
}

template <int DIM, int OP, int WARPS>
void p32_launch(bool split, int blocks, cudaStream_t st, const State& s, const Geometry& g,
                const Consts& k, const BinScratch& b, int self, int reset, int fuse_eos,
                int list_mode) {
  if (split)
    pair32_kernel<DIM, OP, WARPS, true><<<blocks, 32 * WARPS, 0, st>>>(s, g, k, b, self, reset,
                                                                        fuse_eos, list_mode);
  else
    pair32_kernel<DIM, OP, WARPS, false><<<blocks, 32 * WARPS, 0, st>>>(s, g, k, b, self, reset,
                                                                         fuse_eos, list_mode);
}

template <int DIM>
cudaError_t launch_dim(const LaunchCtx& c, const State& s, const Geometry& g, const Consts& k,
                       const BinScratch& b, int cap, int op, int self, int reset, int fuse_eos,
                       int aux_fresh, int list_mode) {
  // a block holds whole items: at least `split` warps
  const int W = std::max(k.warps, k.split);
  const int blocks = (int)(((long long)b.max_items * k.split + W - 1) / W);
  const bool sp = k.split > 1;
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
      if (W == 2) p32_launch<DIM, SPH_OP_DENSITY, 2>(sp, blocks, c.stream, s, g, k, b, self, reset, fuse_eos, 1);
      else if (W == 8) p32_launch<DIM, SPH_OP_DENSITY, 8>(sp, blocks, c.stream, s, g, k, b, self, reset, fuse_eos, 1);
      else p32_launch<DIM, SPH_OP_DENSITY, 4>(sp, blocks, c.stream, s, g, k, b, self, reset, fuse_eos, 1);
      break;
    case SPH_OP_DENSITY_REF:
      if (W == 2) p32_launch<DIM, SPH_OP_DENSITY_REF, 2>(sp, blocks, c.stream, s, g, k, b, self, reset, 0, 1);
      else if (W == 8) p32_launch<DIM, SPH_OP_DENSITY_REF, 8>(sp, blocks, c.stream, s, g, k, b, self, reset, 0, 1);
      else p32_launch<DIM, SPH_OP_DENSITY_REF, 4>(sp, blocks, c.stream, s, g, k, b, self, reset, 0, 1);
      break;
    case SPH_OP_WALL_PRESSURE:
      if (W == 2) p32_launch<DIM, SPH_OP_WALL_PRESSURE, 2>(sp, blocks, c.stream, s, g, k, b, 0, 0, 0, 0);
      else if (W == 8) p32_launch<DIM, SPH_OP_WALL_PRESSURE, 8>(sp, blocks, c.stream, s, g, k, b, 0, 0, 0, 0);
      else p32_launch<DIM, SPH_OP_WALL_PRESSURE, 4>(sp, blocks, c.stream, s, g, k, b, 0, 0, 0, 0);
      break;
    default:
      if (W == 2) p32_launch<DIM, SPH_OP_FORCE, 2>(sp, blocks, c.stream, s, g, k, b, self, reset, 0, list_mode);
      else if (W == 8) p32_launch<DIM, SPH_OP_FORCE, 8>(sp, blocks, c.stream, s, g, k, b, self, reset, 0, list_mode);
      else p32_launch<DIM, SPH_OP_FORCE, 4>(sp, blocks, c.stream, s, g, k, b, self, reset, 0, list_mode);
      break;
  }
  mark(c, kid, 1);
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_fused_pair(const LaunchCtx& c, const FusedBatch& fb, int p, int op, int self,
                              int reset, int fuse_eos, int list_mode) {
  return fb.dim == 2 ? launch_fused_dim<2>(c, fb, p, op, self, reset, fuse_eos, list_mode)
                     : launch_fused_dim<3>(c, fb, p, op, self, reset, fuse_eos, list_mode);
}

cudaError_t launch_pair_mixed(const LaunchCtx& c, const State& s, const Geometry& g,
                              const Consts& k, const BinScratch& b, int cap, int op, int self,
                              int reset, int fuse_eos, int aux_fresh, int lists_valid) {
  if (cap <= 0) return cudaSuccess;
  const int lm = lists_valid ? 2 : 0;
  return k.dim == 2 ? launch_dim<2>(c, s, g, k, b, cap, op, self, reset, fuse_eos, aux_fresh, lm)
                    : launch_dim<3>(c, s, g, k, b, cap, op, self, reset, fuse_eos, aux_fresh, lm);
}

}  // namespace sphgpu
