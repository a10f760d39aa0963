// sph_common.cuh -- device-side data layout and helpers shared by the kernels.
//
// Layout in HBM (struct of arrays, sorted by cell after every binning):
//   x[d], v[d], a[d], xs[d]   double, one array per component (d < DIM)
//   rho, rho_ref, P, Pr       double (Pr = P / rho^2, precomputed per particle)
//   type, rid, cell           int32 (rid = index in the reference's particle
//                             order; cell = 1-based linear cell key)
//   oid                       int64 (index at upload time)
//   pl                        float4: position relative to the origin of the
//                             particle's own cell (FP32) and the type bits in .w
// Two such sets (cur / alt) are ping-ponged by the reorder gather.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace sphgpu {

constexpr int kFluid = 0;
constexpr int kWall = 1;

// device error bits (sticky until read by sph_synchronize)
constexpr int kErrBounds = 1;     // a cell or particle index left its table
constexpr int kErrKeyRange = 2;   // a particle inside the box produced a key outside 1..key_max

struct State {
  double* x[3];
  double* v[3];
  double* a[3];
  double* xs[3];
  double* rho;
  double* rho_ref;
  double* P;
  double* Pr;
  int* type;
  int* rid;
  int* cell;
  long long* oid;
  float4* pl;
  // FP32 neighbour records of the mixed-precision path, 32 bytes per
  // particle, rebuilt every step after the binning (so not ping-ponged):
  // rec[2i] = (cell-relative x, y, z, rho with the sign bit set for walls),
  // rec[2i+1] = (vx, vy, vz, P/rho^2)
  float4* rec;
};

// Cell-table geometry (structs.jl:66-82).  key_max and key_diff fit int32
// (checked when the system is created).
struct Geometry {
  long long key_phase[3];
  long long key_lim[3];
  int key_max;
  int n_diff;
  int key_diff[27];
};

// Constants derived once on the host, with the same expressions as the oracle.
struct Consts {
  double h, inv_h, cw, cr;
  double mass, rho0, B, hdt, dt, eta2, alpha_c0, h_smooth, eps_xsph;
  double gmag, col_height;
  double g[3];
  double dmin[3], dmax[3];
  int vaxis;
  int dim;
  int warps;  // warps per block of the pair passes (2, 4 or 8; tunable)
  // mixed-precision pair passes: warps sharing one work item (1, 2 or 4,
  // i.e. 32, 64 or 128 threads per cell chunk of <= 32 targets; tunable):
  // warp s of an item takes the chunks gi = s, s + split, ... of the
  // neighbour sequence, and the partial sums are added in warp order
  int split;
  // FP32 candidate classification (see the pair kernels): a candidate whose
  // FP32 squared distance lies below s_lo is inside the support, above s_hi
  // outside; in between the FP64 test decides.
  float s_lo, s_hi;
  // the cell size (the support h, or h times the mixed systems' cell factor)
  // and its FP32 copy, of the cell keys, origins and neighbour-cell offsets
  double cell;
  float cellf;
  // the phase of the cell grid per axis: cell i spans [i cell + shift,
  // (i + 1) cell + shift).  0 (the reference's grid) for FP64 systems; 5/16
  // of a cell for mixed ones (not along z in 2D), whose results do not
  // depend on the grid
  double shift[3];
  // mixed systems: 1 / cell, the cell index being floor((x - shift) inv_cell)
  // (a product, where the reference's grid takes a division); 0 for FP64
  // systems.  The key range is computed with the same expression, and the
  // expression is monotone in x, so every point of the box has a key.
  double inv_cell;
  // the largest double s with sqrt_rn(s) <= h: r > h  <=>  fl64(r^2 sum) > s_max
  double s_max;
  // folded constants of the FP64 pair arithmetic: m C_w, m C_r, -(alpha c0) h_smooth
  double mcw, mcr, ca;
  // 5 m C_w and -4 m C_w: m W = t^4 fma(-4 m C_w, t, 5 m C_w)
  double mcw5, mcw4;
  // scale of the positions' fixed-point copies: X = x 2^fx_k, |X| < 2^62
  // over the domain box
  int fx_k;
  // FP32 copies for the mixed-precision pair arithmetic
  float inv_hf, hf, cwf, crf, massf, eta2f, alpha_c0f, h_smoothf, rho0f;
  float gf[3];
  // equation of state (SPH_EOS_*) and the linear one's constants c0^2, rho0^2
  int eos;
  double c2, rho0sq;
};

// One entry of an FP64 target's row (32 bytes, one DRAM sector, written
// whole): the neighbour index (bit 31 set for walls) and up to three values
// -- after the density pass m W, the kernel distance r and t = 1 - r/H (the
// force pass's kernel derivative starts from it), after the force pass the
// pressure factor and the XSPH factor.  A wall's row (its fluid neighbours)
// holds W (without the mass), g.(x_w - x_q) and t for its pressure.
struct __align__(32) RowEntry {
  unsigned long long q;
  double a, b, c;
};

__device__ __forceinline__ void row_store(RowEntry* e, unsigned long long q, double a, double b,
                                          double c = 0.0) {
  asm volatile("st.global.v4.b64 [%0], {%1, %2, %3, %4};" ::"l"(e), "l"(q), "d"(a), "d"(b),
               "d"(c)
               : "memory");
}

// a row entry written by an earlier kernel
__device__ __forceinline__ RowEntry row_load(const RowEntry* e) {
  RowEntry r;
  asm("ld.global.nc.v4.b64 {%0, %1, %2, %3}, [%4];"
      : "=l"(r.q), "=d"(r.a), "=d"(r.b), "=d"(r.c)
      : "l"(e));
  return r;
}

// Scratch of the binning (counting sort by cell key).
// The FP64 force pass's record of one particle (64 bytes, two DRAM sectors,
// rebuilt before every force pass from the SoA state, sph_tile64.cu): what
// the force kernels gather per neighbour -- the fixed-point position copies
// (fx_fix; X[2] = 0 in 2D), the velocity, the density and P/rho^2 -- in two
// 256-bit loads instead of eleven scalar ones.
struct __align__(64) FxRec {
  long long X[3];
  double v0;
  double v1, v2, rho, pr;
};

struct BinScratch {
  int* keys;        // per particle (storage order before the sort)
  int* slots;       // rank of the particle inside its cell's bucket (atomic)
  int* counts;      // key_max + 3 bucket counts
  int* cell_start;  // key_max + 3 exclusive prefix sums of counts
  int* perm_tmp;    // bucketed old index
  int* rid_tmp;     // bucketed reference index (after removal remap)
  int* perm;        // final old index for every new slot
  int* rid_sorted;  // final reference index for every new slot
  int* flag_by_rid; // removal flags indexed by reference index
  int* rem_list;    // removed reference indices, ascending
  int* ident;       // identity permutation used by the tail-fill replay
  int* moved_to;    // new reference index of a survivor moved from the tail
  int* inv_rid;     // storage index of every reference index
  int* d_n;         // particle count (device-resident)
  int* d_nrem;      // particles removed by the last binning
  int* d_err;       // error bits
  int* scan_tmp;    // block sums of the scans over the cell tables
  int* pscan_tmp;   // block sums of the scans over the particles (FP64 rows)
  unsigned long long* d_pairs;
  // hits per category: [0] density sums, [1] wall pressure (fluid q),
  // [2] force fluid-fluid, [3] force fluid-wall, [4] force with viscosity
  unsigned long long* d_cat;
  // pair-pass work list: one item per group of <= 32 targets of one cell
  int2* items;      // (first target, count)
  int* item_off;    // key_max + 3: exclusive prefix of items per cell
  int max_items;    // capacity of `items`
  // FP64 passes (null in mixed-precision systems).  Compact rows (CSR):
  // particle i's row -- its neighbours in the reference's order; a wall's
  // row holds its fluid neighbours -- is hit_count[i] entries starting at
  // entry 4 * row_base[i] of `rows` (every row padded to a multiple of four
  // entries, 128 bytes).  The row is split into one segment per
  // neighbour-cell slot c (key_diff order): the tile kernel counts each
  // segment's hits into rseg[c * rseg_stride + i] (slot-major, so that the
  // passes over the particles read and write it coalesced), the row count
  // turns the counts into the segments' first entries relative to the row's
  // start and the offsets pass adds the start 4 row_base[i] (sph_tile64.cu).
  // A row that cannot be used (a segment of more than kSegMax hits, a
  // neighbour cell of more than 65535 particles) has hit_count kRowOver and its target
  // traverses; so does every target when the rows do not fit row_cap (the
  // host grows them before the next pass).
  RowEntry* rows;
  long long row_cap;    // entries `rows` holds (< 2^32)
  unsigned* row_base;   // cap + 1: exclusive prefix of c4 (row starts / 4)
  int* c4;              // cap + 1: (hit_count + 3) / 4, 0 for rows not used
  unsigned* rseg;       // n_diff per particle: hits per slot, then first entries
  int rseg_stride;      // particles per slot of rseg (the arena's capacity)
  int* hit_count;
  // the largest row total a pass needed beyond row_cap (host-mapped memory,
  // read by the host to grow the rows between passes)
  unsigned long long* need_host;
  long long* xfix[3];  // positions as exact fixed-point integers (fx_fix), per step
  FxRec* frec;         // per particle, for the force pass (FxRec)
  // the traversal's per-lane hit lists (sph_cellwarp.cuh): trav_slots warps,
  // each 32 lists of kTravCap entries, claimed by a persistent grid's warps
  int* trav;
  int trav_slots;
  int* work_ctr;       // the traversal's item counter (reset before each launch)
  // the step's unordered pairs (sph_tile64.cu), pair_cap at most: the two
  // particles and (rank in p's segment, rank in q's segment, slot, walls)
  int* pair_p;
  int* pair_q;
  unsigned* pair_m;
  long long pair_cap;
  unsigned long long* d_npairs;  // pairs listed (may exceed pair_cap)
  // the list (or the rows) overflowed: every target traverses
  int* d_pover;
  int* d_rover;                  // some target's row overflowed (it traverses)
  // the sum of c4 over the particles in 64 bits (follows d_rover: cleared
  // with the pair count and the flags), so that an int32 scan that wrapped
  // is never trusted
  unsigned long long* d_rowsum;
  // walls of the current cells (the density pass's row count lists them):
  // wall_list[0 .. d_nwall[0]) the walls with fluid neighbours in their rows,
  // wall_list[cap - 1 - j], j < d_nwall[1], the walls without (follows
  // d_rowsum: cleared with it)
  int* d_nwall;
  int* wall_list;
  int wall_cap;
  int* cell_fluid;    // key_max + 3: fluid particles per cell
  // mixed-precision passes: one 32-bit hit mask per lane and 32-candidate
  // chunk of the neighbour sequence (sph_pair32.cu); item j of cell k owns
  // the slots chunk_off[k] + j * n_k .. + n_k, n_k = the chunks of k's
  // neighbour cells (null in FP64 systems)
  unsigned* ck_mask;  // ck_cap * 32
  int ck_cap;
  int* chunk_off;     // key_max + 3: exclusive prefix of the cells' slots
};

constexpr int kSegMax = 1022;        // hits of one row segment a rank can address
constexpr int kRowOver = 0x7fffffff; // hit_count of a row that is not used
constexpr unsigned kNoRow = 0xffffffffu;
constexpr int kTravCap = 256;        // entries of a traversal hit list

__host__ __device__ __forceinline__ size_t rseg_at(const BinScratch& b, int i, int c) {
  return (size_t)c * (size_t)b.rseg_stride + (size_t)i;
}

// Upper bound of the work-list length for n particles (every cell with
// particles contributes ceil(c/32) <= c/32 + 1 items).
inline int max_work_items(int n, int key_max) {
  const long long b = (long long)n / 32 + (long long)(n < key_max ? n : key_max) + 2;
  return (int)b;
}

constexpr int kCatDensity = 0;
constexpr int kCatWall = 1;
constexpr int kCatForceFluid = 2;
constexpr int kCatForceWall = 3;
constexpr int kCatForceAV = 4;
constexpr int kNumCat = 8;

__device__ __forceinline__ void decode_key(const Geometry& g, int key, int& cx, int& cy, int& cz) {
  const int k0 = key - 1;
  const int l0 = (int)g.key_lim[0];
  const int l1 = (int)g.key_lim[1];
  cx = k0 % l0;
  const int t = k0 / l0;
  cy = t % l1;
  cz = t / l1;
}

// v < 0.0 exactly (false for -0 and NaN), on the integer pipe
__device__ __forceinline__ bool lt0(double v) {
  const long long b = __double_as_longlong(v);
  const long long m = b & 0x7FFFFFFFFFFFFFFFLL;
  return b < 0 && m != 0 && m <= 0x7FF0000000000000LL;
}

// ---- FP64 square root and reciprocal on the integer pipes ----------------
// GB300's FP64 pipe issues 2 operations per SM per clock and a correctly
// rounded square root or reciprocal takes ~7.5 / ~4.6 of them; the same
// results are formed here with integer instructions (the pipes the FP64
// passes leave idle), for positive normal inputs with normal results
// (anything else takes the FP64 operation out of line):
//   sqrt: s = M 2^e (M of 53 bits), e made even, sqrt(s) = sqrt(N) 2^(e/2 - 26)
//     with N = M' 2^52 in [2^104, 2^106), so Q = floor(sqrt N) has 53 bits;
//   1/y = (2^105 / M) 2^(-e-105), Q = floor(2^105 / M) of 53 bits.
// Q comes from an FP32 seed (rsqrt / rcp approximations) and two Newton
// corrections in 128-bit integers, is adjusted to the exact floor (one step
// at most; the floor condition is then verified exactly) and rounded to
// nearest with the exact remainder (even on a tie).  The method is the
// textbook one: Newton-Raphson iteration for the reciprocal and the
// reciprocal square root (Markstein, IBM J. Res. Dev. 34(1), 1990), carried
// out in integer arithmetic, followed by correct rounding decided from the
// exact remainder N - Q^2 or 2^105 - Q M (Muller et al., Handbook of
// Floating-Point Arithmetic, 2nd ed. 2018, the chapters on division and
// square root by iteration).  No library routine's constants or steps are
// reproduced; tests compare every result with the IEEE operation.
static __device__ __noinline__ double isqrt_fallback(double s) { return sqrt(s); }
static __device__ __noinline__ double ircp_fallback(double y) { return __drcp_rn(y); }

// f 2^scale as an integer (f positive and normal, the result below 2^63)
__device__ __forceinline__ unsigned long long f32_fix(float f, int scale) {
  const unsigned b = __float_as_uint(f);
  const int sh = (int)(b >> 23) - 150 + scale;
  const unsigned long long m = (unsigned long long)((b & 0x7fffffu) | 0x800000u);
  return sh >= 0 ? m << sh : m >> -sh;
}

// RN(sqrt(s))
__device__ __forceinline__ double isqrt_rn(double s) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(s);
  const int E = (int)(b >> 52);  // the sign bit makes a negative input's E >= 0x800
  if (E <= 0 || E >= 0x7ff) return isqrt_fallback(s);
  const unsigned long long M = (b & 0xfffffffffffffull) | (1ull << 52);
  const int e = E - 1075;
  const int odd = e & 1;
  const unsigned long long M2 = M << odd;  // [2^52, 2^54)
  const int e2 = e - odd;
  const unsigned __int128 N = (unsigned __int128)M2 << 52;
  // the seed: u = M2 / 2^52 in [1, 4) from the leading bits
  const float u = __uint_as_float((M2 >> 53) ? (128u << 23) | (unsigned)((M2 >> 30) & 0x7fffffu)
                                             : (127u << 23) | (unsigned)((M2 >> 29) & 0x7fffffu));
  float y0;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y0) : "f"(u));
  unsigned long long q = f32_fix(u * y0, 52);  // ~ sqrt(N)
  const long long Y = (long long)f32_fix(y0, 31);
#pragma unroll
  for (int it = 0; it < 2; ++it) {
    // q += (N - q^2) / (2 q), with 1/(2q) ~ y0 2^-53
    const __int128 D = (__int128)(N - (unsigned __int128)q * q);
    q = (unsigned long long)((long long)q + (long long)(((D >> 22) * Y) >> 62));
  }
  unsigned __int128 q2 = (unsigned __int128)q * q;
  if (q2 > N) {
    --q;
    q2 = (unsigned __int128)q * q;
  } else if (N - q2 > 2 * (unsigned __int128)q) {
    ++q;
    q2 = (unsigned __int128)q * q;
  }
  if (q2 > N || N - q2 > 2 * (unsigned __int128)q) return isqrt_fallback(s);
  if (N - q2 > q) ++q;  // sqrt(N) >= q + 1/2  <=>  N - q^2 > q (never a tie)
  return __longlong_as_double((long long)(((unsigned long long)(e2 / 2 - 26 + 1074) << 52) + q));
}

// RN(1/y)
__device__ __forceinline__ double ircp_rn(double y) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(y);
  const int E = (int)(b >> 52);
  if (E <= 1 || E >= 2045) return ircp_fallback(y);  // keeps 1/y normal
  const unsigned long long M = (b & 0xfffffffffffffull) | (1ull << 52);
  const int e = E - 1075;
  const unsigned __int128 T = (unsigned __int128)1 << 105;
  const float u = __uint_as_float((127u << 23) | (unsigned)((M >> 29) & 0x7fffffu));  // [1, 2)
  float y0;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y0) : "f"(u));
  unsigned long long q = f32_fix(y0, 53);  // ~ 2^105 / M
  const long long Y = (long long)f32_fix(y0, 31);
#pragma unroll
  for (int it = 0; it < 2; ++it) {
    // q += (2^105 - q M) / M, with 1/M ~ y0 2^-52
    const __int128 D = (__int128)(T - (unsigned __int128)q * M);
    q = (unsigned long long)((long long)q + (long long)(((D >> 22) * Y) >> 61));
  }
  unsigned __int128 qm = (unsigned __int128)q * M;
  if (qm > T) {
    --q;
    qm -= M;
  } else if (T - qm >= M) {
    ++q;
    qm += M;
  }
  if (qm > T || T - qm >= M) return ircp_fallback(y);
  const unsigned __int128 R2 = 2 * (T - qm);
  if (R2 > M || (R2 == M && (q & 1ull))) ++q;
  return __longlong_as_double((long long)(((unsigned long long)(-e - 105 + 1074) << 52) + q));
}

// 2.0 / y, correctly rounded: 2 RN(1/y) with the factor 2 applied to the
// exponent field, which is exact while RN(1/y) and its double are normal;
// otherwise the division itself
__device__ __forceinline__ double two_over(double y) {
  const double r = ircp_rn(y);
  const long long b = __double_as_longlong(r);
  const long long e = (b >> 52) & 0x7FF;
  return (e >= 1 && e <= 0x7FD) ? __longlong_as_double(b + (1LL << 52)) : __ddiv_rn(2.0, y);
}

// The Wendland quintic and its derivative over r (kernels.jl:108-195, which
// are @fastmath) in the one evaluation order the CPU restatement also uses:
// t = 1 - r (1/h) as one fused operation, 0 beyond the support,
// W = (C_w t^4)(5 - 4t) (5 - 4t = 1 + 4x), rDW = C_r t^3.
__device__ __forceinline__ double ker_t(const Consts& k, double r) {
  const double t = __fma_rn(-r, k.inv_h, 1.0);
  return lt0(t) ? 0.0 : t;
}
__device__ __forceinline__ double ker_w(const Consts& k, double r) {
  const double t = ker_t(k, r);
  const double t2 = t * t;
  return (k.cw * (t2 * t2)) * __fma_rn(-4.0, t, 5.0);
}
__device__ __forceinline__ double ker_rdw(const Consts& k, double r) {
  const double t = ker_t(k, r);
  return k.cr * ((t * t) * t);
}

// The equation of state of a fluid particle and the pressure term of the
// force, P/rho^2 (Tait, the dam-break scheme; B = c0^2 rho0 / 7, ^7 as a
// product chain) or P/rho0^2 (the linear P = c^2 (rho - rho0) of
// tests/test_collision_2d.jl:71-78), in the oracle's evaluation order.
__device__ __forceinline__ void eos_eval(const Consts& k, double rho, double rho_ref, double& P,
                                         double& Pr) {
  if (k.eos == 1) {
    P = k.c2 * (rho - rho_ref);
    Pr = P / k.rho0sq;
  } else {
    const double ratio = rho / rho_ref;
    const double r2 = ratio * ratio;
    const double r4 = r2 * r2;
    const double r7 = (r4 * r2) * ratio;
    P = k.B * (r7 - 1.0);
    Pr = P / (rho * rho);
  }
}

// x in cell units along axis d: the reference's (x - 0) / h for FP64
// systems, a product with 1/cell for mixed ones (Consts.inv_cell)
__device__ __forceinline__ double cell_coord(const Consts& k, double x, int d) {
  const double u = __dsub_rn(x, k.shift[d]);
  return k.inv_cell != 0.0 ? __dmul_rn(u, k.inv_cell) : __ddiv_rn(u, k.cell);
}

// structs.jl:97-106 for an arbitrary point: -1 when a coordinate is NaN,
// infinite or outside the Int64 range (the reference's try/catch).
__device__ __forceinline__ long long find_key_point(const Geometry& g, const Consts& k,
                                                    const double x[3]) {
  long long ijk[3];
  for (int d = 0; d < 3; ++d) {
    const double f = floor(cell_coord(k, x[d], d));
    if (!(f >= -9223372036854775808.0 && f < 9223372036854775808.0)) return -1;
    ijk[d] = 1 + (long long)f - g.key_phase[d];
  }
  return ijk[0] + g.key_lim[0] * (ijk[1] - 1) + g.key_lim[0] * g.key_lim[1] * (ijk[2] - 1);
}

// The reference's distance test, r = sqrt((d1*d1 + d2*d2) + d3*d3) and
// r > h (core.jl:8-10, :105; algebra.jl:49-60), with round-to-nearest
// intrinsics so that no compiler contraction can change a rounding: the
// FP64 band test gives the same answer in every translation unit.  Because
// the correctly rounded square root is monotone, sqrt_rn(s) > h exactly when
// s > s_max, so no square root is taken.
template <int DIM>
__device__ __forceinline__ bool within_rn(const State& s, const Consts& k, const double* xp, int q) {
  const double d0 = __dsub_rn(xp[0], __ldg(&s.x[0][q]));
  const double d1 = __dsub_rn(xp[1], __ldg(&s.x[1][q]));
  double ss = __dadd_rn(__dmul_rn(d0, d0), __dmul_rn(d1, d1));
  if (DIM == 3) {
    const double d2 = __dsub_rn(xp[2], __ldg(&s.x[2][q]));
    ss = __dadd_rn(ss, __dmul_rn(d2, d2));
  }
  return !(ss > k.s_max);
}

// Exact position differences on the integer pipes.  GB300 executes FP64
// arithmetic and int64 <-> FP64 conversions on one slow pipe, so the
// separations x_p - x_q of the FP64 pair passes are formed from fixed-point
// copies X = x 2^k: D = X_p - X_q is the exact difference in units of 2^-k,
// and RN(D) 2^-k = RN(x_p - x_q) is the correctly rounded FP64 subtraction
// (scaling by a power of two commutes with rounding in the normal range).
// A position without an exact copy (|x| below 2^(52-k), -0, subnormal or
// out of range) takes the FP64 subtraction.
constexpr long long kFxNone = (long long)0x8000000000000000ull;

__device__ __forceinline__ long long fx_fix(double x, int k) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const int E = (int)((b >> 52) & 0x7ff);
  if (E == 0) return b == 0ull ? 0 : kFxNone;  // +0 is exact; -0 and subnormals are not
  if (E == 0x7ff) return kFxNone;
  const unsigned long long m = (b & 0xfffffffffffffull) | (1ull << 52);
  const int t = E - 1075 + k;
  unsigned long long X;
  if (t >= 0) {
    if (t > 9) return kFxNone;  // |X| >= 2^62
    X = m << t;
  } else {
    if (t < -52 || (m & ((1ull << -t) - 1ull)) != 0ull) return kFxNone;  // not a multiple of 2^-k
    X = m >> -t;
  }
  return (b >> 63) ? -(long long)X : (long long)X;
}

// RN(X_p - X_q) 2^-k as a double (ties to even), both copies exact
__device__ __forceinline__ double fx_diff(long long Xp, long long Xq, int k) {
  const long long D = Xp - Xq;
  if (D == 0) return 0.0;
  const unsigned long long neg = (unsigned long long)(D >> 63);
  const unsigned long long a = ((unsigned long long)D ^ neg) - neg;
  const int L = 63 - __clzll((long long)a);  // the leading one
  unsigned long long m;
  if (L <= 52) {
    m = a << (52 - L);
  } else {
    const int sh = L - 52;
    m = a >> sh;
    const unsigned long long rem = a & ((1ull << sh) - 1ull), half = 1ull << (sh - 1);
    m += (rem > half || (rem == half && (m & 1ull))) ? 1ull : 0ull;
  }
  // m holds the leading one at bit 52 (or 2^53 after rounding up): adding it
  // to the exponent field one below the leading one's places it exactly
  return __longlong_as_double((long long)((neg & 0x8000000000000000ull) +
                                          ((unsigned long long)(L - k + 1022) << 52) + m));
}

// The FP64 subtraction for positions without exact copies, out of line so
// that it is not evaluated speculatively beside the integer path.
static __device__ __noinline__ double fx_fallback(double xp, const double* xq) { return xp - __ldg(xq); }

// x_p - x_q along axis d, with p's own copy Xp and position xp at hand
__device__ __forceinline__ double fx_sep1(long long Xp, const double* xp, const State& s,
                                          const long long* const* xfix, int k, int d, int q) {
  const long long Xq = __ldg(&xfix[d][q]);
  if (Xp == kFxNone || Xq == kFxNone) return fx_fallback(__ldg(xp), &s.x[d][q]);
  return fx_diff(Xp, Xq, k);
}

// x_p - x_q along axis d from both copies at hand (xp, xq: the positions,
// read only when a copy is missing)
__device__ __forceinline__ double fx_sep2(long long Xp, const double* xp, long long Xq,
                                          const double* xq, int k) {
  if (Xp == kFxNone || Xq == kFxNone) return fx_fallback(__ldg(xp), xq);
  return fx_diff(Xp, Xq, k);
}

// The two halves of a force record (one 256-bit load each).
__device__ __forceinline__ void frec_load_x(const FxRec* r, long long& X0, long long& X1,
                                            long long& X2, double& v0) {
  asm("ld.global.nc.v4.b64 {%0, %1, %2, %3}, [%4];"
      : "=l"(X0), "=l"(X1), "=l"(X2), "=d"(v0)
      : "l"(r));
}
__device__ __forceinline__ void frec_load_v(const FxRec* r, double& v1, double& v2, double& rho,
                                            double& pr) {
  asm("ld.global.nc.v4.b64 {%0, %1, %2, %3}, [%4];"
      : "=d"(v1), "=d"(v2), "=d"(rho), "=d"(pr)
      : "l"(&r->v1));
}

__device__ __forceinline__ void frec_load_v12(const FxRec* r, double& v1, double& v2) {
  asm("ld.global.nc.v2.f64 {%0, %1}, [%2];" : "=d"(v1), "=d"(v2) : "l"(&r->v1));
}

// x_p - x_q along axis d: from the fixed-point copies when both are exact
__device__ __forceinline__ double fx_sep(const State& s, const long long* const* xfix, int k,
                                         int d, int p, int q) {
  return fx_sep1(__ldg(&xfix[d][p]), &s.x[d][p], s, xfix, k, d, q);
}

// Two FP32 lanes per 64-bit register (Blackwell's packed FP32 arithmetic).
__device__ __forceinline__ unsigned long long f2_pack(float lo, float hi) {
  return (unsigned long long)__float_as_uint(lo) | ((unsigned long long)__float_as_uint(hi) << 32);
}
__device__ __forceinline__ unsigned long long f2_sub(unsigned long long a, unsigned long long b) {
  unsigned long long r;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ unsigned long long f2_add(unsigned long long a, unsigned long long b) {
  unsigned long long r;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ unsigned long long f2_mul(unsigned long long a, unsigned long long b) {
  unsigned long long r;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ unsigned long long f2_fma(unsigned long long a, unsigned long long b,
                                                     unsigned long long c) {
  unsigned long long r;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
  return r;
}

__device__ __forceinline__ unsigned lanemask_lt() {
  unsigned m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

}  // namespace sphgpu
