// sph_api.cu -- the C ABI (include/sphgpu.h): handle, device memory, stream,
// argument checking and the order of kernel launches for each call.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "sph_launch.h"
#include "sph_system.h"
#include "sphgpu.h"

using namespace sphgpu;

// Many systems stepped together: each member's fused step is captured once
// into a CUDA graph as an independent branch (two steps per graph, so every
// member's ping-pong buffers end where they started) and the graph is
// replayed; the branches overlap on the device.
struct sph_batch {
  std::vector<sph_system*> members;
  std::vector<long long> generations;
  // each member's current particle set (x of its `cur` ping-pong half) when
  // the graph was captured: a graph of two steps starts from that half, so
  // after an odd number of steps taken outside it the graph is stale
  std::vector<const double*> cur0;
  int device = 0;
  cudaStream_t origin = nullptr;
  cudaEvent_t fork = nullptr;
  cudaEvent_t after = nullptr;
  std::vector<cudaEvent_t> joins;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  long long kernels_per_graph = 0;
  long long launches = 0;
  long long graph_launches = 0;
  std::string err;
  // fused mode (mixed-precision members of one dimension): every kernel of
  // the step is one launch over all members
  bool fusable = false;
  bool fused = false;
  int fused_warps = 4;  // warps per block of the fused pair passes
  void* fdev = nullptr;  // device copy of the member arguments and block tables
  long long counted = 0;  // kernels counted while capturing
};

namespace {

int fail(sph_system* s, int code, const char* fmt, ...) {
  if (s) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    s->err = buf;
  }
  return code;
}

#define CK(call)                                                                      \
  do {                                                                                \
    cudaError_t e_ = (call);                                                          \
    if (e_ != cudaSuccess)                                                            \
      return fail(s, SPH_ERR_CUDA, "%s failed: %s", #call, cudaGetErrorString(e_));   \
  } while (0)

cudaEvent_t get_event(sph_system* s) {
  if (!s->pool.empty()) {
    cudaEvent_t e = s->pool.back();
    s->pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

void hook(void* owner, int kid, int phase, int kernels) {
  sph_system* s = (sph_system*)owner;
  if (phase == 0) {
    if (s->profiling) {
      s->open_start = get_event(s);
      cudaEventRecord(s->open_start, s->stream);
    }
    return;
  }
  s->kernel_launches[kid] += kernels;
  s->total_launches += kernels;
  if (s->profiling && s->open_start) {
    cudaEvent_t stop = get_event(s);
    cudaEventRecord(stop, s->stream);
    s->pending.push_back({kid, s->open_start, stop});
    s->open_start = nullptr;
  }
}

LaunchCtx ctx(sph_system* s) { return LaunchCtx{s->stream, s, hook}; }

int flush_profile(sph_system* s) {
  if (s->pending.empty()) return SPH_OK;
  CK(cudaStreamSynchronize(s->stream));
  for (auto& p : s->pending) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, p.start, p.stop);
    s->total_ms[p.kid] += ms;
    s->pool.push_back(p.start);
    s->pool.push_back(p.stop);
  }
  s->pending.clear();
  return SPH_OK;
}

size_t align_up(size_t v) { return (v + 255) & ~(size_t)255; }

// Carves the arena for capacity C.  With base == nullptr only the size is
// computed.
size_t carve(sph_system* s, char* base, size_t C) {
  size_t off = 0;
  auto take = [&](size_t bytes) -> void* {
    void* p = base ? base + off : nullptr;
    off += align_up(bytes);
    return p;
  };
  const int D = s->params.dim;
  State* sets[2] = {&s->cur, &s->alt};
  for (State* st : sets) {
    for (int d = 0; d < 3; ++d) {
      const bool use = d < D;
      st->x[d] = use ? (double*)take(8 * C) : nullptr;
      st->v[d] = use ? (double*)take(8 * C) : nullptr;
      st->a[d] = use ? (double*)take(8 * C) : nullptr;
      st->xs[d] = use ? (double*)take(8 * C) : nullptr;
    }
    st->rho = (double*)take(8 * C);
    st->rho_ref = (double*)take(8 * C);
    st->P = (double*)take(8 * C);
    st->Pr = (double*)take(8 * C);
    st->type = (int*)take(4 * C);
    st->rid = (int*)take(4 * C);
    st->cell = (int*)take(4 * C);
    st->oid = (long long*)take(8 * C);
    st->pl = (float4*)take(16 * C);
  }
  s->cur.rec = s->alt.rec =
      s->params.precision == SPH_PREC_MIXED ? (float4*)take(32 * C) : nullptr;
  BinScratch& b = s->b;
  b.keys = (int*)take(4 * C);
  b.slots = (int*)take(4 * C);
  b.perm_tmp = (int*)take(4 * C);
  b.rid_tmp = (int*)take(4 * C);
  b.perm = (int*)take(4 * C);
  b.rid_sorted = (int*)take(4 * C);
  b.flag_by_rid = (int*)take(4 * C);
  b.rem_list = (int*)take(4 * C);
  b.ident = (int*)take(4 * C);
  b.moved_to = (int*)take(4 * C);
  b.inv_rid = (int*)take(4 * C);
  b.max_items = max_work_items((int)C, s->geo.key_max);
  b.items = (int2*)take(8 * (size_t)b.max_items);
  if (s->params.precision == SPH_PREC_MIXED) {
    // hit masks: a full 3D item (32 targets, cells of ~64 particles) has 54
    // chunks, ~1.7 per particle; 2D items ~0.4 per particle.  Items beyond
    // the capacity traverse in the force pass too.
    const long long cap = 2LL * (long long)C + 64;
    b.ck_cap = (int)(cap < 0x3ffffffLL * 16 ? cap : 0x3ffffffLL * 16);
    b.ck_mask = (unsigned*)take(4 * 32 * (size_t)b.ck_cap);
    b.hit_count = nullptr;
    b.wall_list = nullptr;
    b.wall_cap = 0;
    b.row_base = nullptr;
    b.c4 = nullptr;
    b.rseg = nullptr;
    b.pscan_tmp = nullptr;
    b.xfix[0] = b.xfix[1] = b.xfix[2] = nullptr;
    b.frec = nullptr;
    b.trav = nullptr;
    b.trav_slots = 0;
  } else {
    // the rows themselves and the pair list are sized from the counts and
    // live in their own allocation (ensure_rows); per particle here: the
    // row length and start, the per-slot segment offsets, the positions'
    // fixed-point copies and the force records
    b.hit_count = (int*)take(4 * C);
    b.wall_list = (int*)take(4 * C);
    b.wall_cap = (int)C;
    b.row_base = (unsigned*)take(4 * (C + 1));
    b.c4 = (int*)take(4 * (C + 1));
    b.pscan_tmp = (int*)take(4 * (scan_tmp_ints((int)C + 1) + 64));
    for (int d = 0; d < 3; ++d) b.xfix[d] = d < D ? (long long*)take(8 * C) : nullptr;
    b.frec = (FxRec*)take(sizeof(FxRec) * C);  // 256-byte aligned start
    b.rseg = (unsigned*)take(4 * (size_t)s->geo.n_diff * C);
    b.rseg_stride = (int)C;
    // the traversal's hit lists: one slot per warp of its persistent grid,
    // about one warp per 32 particles up to a full device (64 warps per SM)
    b.trav_slots = (int)std::min<size_t>(C / 32 + 64, 64 * (size_t)s->sms);
    b.trav = (int*)take(4 * (size_t)b.trav_slots * 32 * kTravCap);
    b.ck_cap = 0;
    b.ck_mask = nullptr;
  }
  // host-transfer staging: 72 bytes per particle (x, v, rho, rho_ref,
  // type of an upload); the debug listings put 4 + 8 bytes per particle at a
  // 256-byte boundary, which the 512 bytes of slack cover for any C
  s->staging = take(72 * C + 512);
  return off;
}

int ensure_capacity(sph_system* s, int n) {
  if (n <= s->cap && s->arena) return SPH_OK;
  if (s->arena) {
    CK(cudaStreamSynchronize(s->stream));
    CK(cudaFree(s->arena));
    s->arena = nullptr;
    s->cap = 0;
  }
  const size_t C = (size_t)(n > 0 ? n : 1);
  const size_t bytes = carve(s, nullptr, C);
  void* p = nullptr;
  if (cudaMalloc(&p, bytes) != cudaSuccess) {
    cudaGetLastError();
    return fail(s, SPH_ERR_NOMEM, "cannot allocate %zu bytes of device memory for %d particles",
                bytes, n);
  }
  s->arena = p;
  carve(s, (char*)p, C);
  s->cap = (int)C;
  ++s->generation;
  return SPH_OK;
}

// Rows beyond this many entries cannot be addressed by the 32-bit segment
// offsets; such systems keep the traversal.
constexpr unsigned long long kMaxRowEntries = 0xffffffffull - 8191ull;

bool capturing(sph_system* s) {
  cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(s->stream, &st) != cudaSuccess) {
    cudaGetLastError();
    return true;  // be safe: no allocation
  }
  return st != cudaStreamCaptureStatusNone;
}

// The rows and pair list for `need` row entries: reallocated (nothing to
// keep: every density pass rewrites them) with 1/12 headroom, so that the
// slow growth of a compressing flow does not overflow every few steps.
// Changes the launch arguments, so captured graphs are recaptured.
int ensure_rows(sph_system* s, unsigned long long need) {
  BinScratch& b = s->b;
  if ((long long)need <= b.row_cap || s->rows_impossible) return SPH_OK;
  if (need > kMaxRowEntries) {
    s->rows_impossible = true;
    return SPH_OK;
  }
  CK(cudaStreamSynchronize(s->stream));
  if (s->rowbuf) CK(cudaFree(s->rowbuf));
  s->rowbuf = nullptr;
  s->rowbuf_bytes = 0;
  b.rows = nullptr;
  b.row_cap = 0;
  b.pair_p = b.pair_q = nullptr;
  b.pair_m = nullptr;
  b.pair_cap = 0;
  ++s->generation;
  unsigned long long cap = need + need / 12 + 4096;
  cap = std::min(cap, kMaxRowEntries) & ~3ull;
  // a listed pair fills two row entries (fluid-fluid: both targets;
  // fluid-wall: the fluid target and the wall's row), so half the entries
  // bound the pairs
  const unsigned long long pcap = cap / 2 + 1024;
  const size_t bytes = align_up(sizeof(RowEntry) * cap) + 3 * align_up(4 * pcap);
  void* p = nullptr;
  if (cudaMalloc(&p, bytes) != cudaSuccess) {
    cudaGetLastError();
    return fail(s, SPH_ERR_NOMEM, "cannot allocate %zu bytes for the FP64 rows (%llu entries)",
                bytes, cap);
  }
  char* c = (char*)p;
  b.rows = (RowEntry*)c;
  c += align_up(sizeof(RowEntry) * cap);
  b.pair_p = (int*)c;
  c += align_up(4 * pcap);
  b.pair_q = (int*)c;
  c += align_up(4 * pcap);
  b.pair_m = (unsigned*)c;
  b.row_cap = (long long)cap;
  b.pair_cap = (long long)pcap;
  s->rowbuf = p;
  s->rowbuf_bytes = bytes;
  return SPH_OK;
}

// Grows the rows to what an earlier pass reported it needed (the host-mapped
// word); never during a stream capture.  `wait`: first let the stream finish,
// so that the report of passes just queued is seen.  Callers: before a
// density pass or a step (which rebuild the rows), or right after a density
// pass that had no rows (its wall-pressure and force passes traverse).
int grow_rows(sph_system* s, bool wait) {
  if (s->params.precision == SPH_PREC_MIXED || !s->need_host || s->rows_impossible) return SPH_OK;
  if (capturing(s)) return SPH_OK;
  if (wait) CK(cudaStreamSynchronize(s->stream));
  volatile unsigned long long* need = s->need_host;
  const unsigned long long v = *need;
  if ((long long)v <= s->b.row_cap) return SPH_OK;
  const int rc = ensure_rows(s, v);
  *need = 0;
  return rc;
}

int read_count(sph_system* s, int* n) {
  CK(cudaMemcpyAsync(n, s->b.d_n, sizeof(int), cudaMemcpyDeviceToHost, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  s->n_host = *n;
  return SPH_OK;
}

int pair_pass(sph_system* s, int op, int self, int reset, int fuse_eos) {
  // the rows may be replaced only where a pass rebuilds them: before a
  // density pass (the wall-pressure and force passes read what it wrote)
  int rc = SPH_OK;
  if (op == SPH_OP_DENSITY || op == SPH_OP_DENSITY_REF) {
    rc = grow_rows(s, false);
    if (rc) return rc;
  }
  cudaError_t e;
  if (s->params.precision == SPH_PREC_MIXED) {
    // the wall pressure reads fluid records, the force every record
    const bool fresh = op == SPH_OP_FORCE           ? s->aux_fluid && s->aux_wall
                       : op == SPH_OP_WALL_PRESSURE ? s->aux_fluid
                                                    : true;
    e = launch_pair_mixed(ctx(s), s->cur, s->geo, s->k, s->b, s->n_host, op, self, reset, fuse_eos,
                          fresh ? 1 : 0, s->lists_valid ? 1 : 0);
    if (!fresh && e == cudaSuccess) s->aux_fluid = s->aux_wall = true;  // rebuilt first
  } else {
    e = launch_pair_fp64(ctx(s), s->cur, s->geo, s->k, s->b, s->n_host, op, self, reset, fuse_eos,
                         s->lists_valid ? 1 : 0);
  }
  if (e == cudaErrorNotSupported)
    return fail(s, SPH_ERR_UNSUPPORTED, "pair operator %d is not provided in this precision", op);
  if (e != cudaSuccess) return fail(s, SPH_ERR_CUDA, "pair pass launch: %s", cudaGetErrorString(e));
  // a fused density pass leaves the fluid records current; a non-fused one
  // changes rho without P, so they are stale; the wall pressure writes the
  // walls' records
  if (op == SPH_OP_DENSITY) s->aux_fluid = fuse_eos != 0;
  if (op == SPH_OP_WALL_PRESSURE) s->aux_wall = true;
  // the density passes keep the hit masks (mixed) or the rows (FP64) for the
  // force pass of the same binning; an FP64 force pass turns the rows' m W
  // into its own factors (a traversing pass only writes the rows of targets
  // that have none: passes without valid rows, overflowed rows)
  if (op == SPH_OP_DENSITY || op == SPH_OP_DENSITY_REF) {
    s->lists_valid = true;
    s->hits_valid = true;
    // the first density pass of an FP64 system finds the rows' size (it
    // traverses, having none): allocate them before the next pass
    if (s->params.precision != SPH_PREC_MIXED && s->b.row_cap == 0) {
      rc = grow_rows(s, true);
      if (rc) return rc;
    }
  }
  else if (op == SPH_OP_FORCE && s->params.precision != SPH_PREC_MIXED)
    s->lists_valid = false;
  return SPH_OK;
}

int binning(sph_system* s, int step_mode, int gather_mode) {
  cudaError_t e = launch_binning(ctx(s), s->cur, s->alt, s->geo, s->k, s->b, s->n_host, step_mode,
                                 gather_mode);
  if (e != cudaSuccess) return fail(s, SPH_ERR_CUDA, "binning launch: %s", cudaGetErrorString(e));
  std::swap(s->cur, s->alt);
  s->cells_valid = true;
  s->aux_fluid = s->aux_wall = false;
  s->lists_valid = false;
  s->hits_valid = false;
  return SPH_OK;
}

int unary(sph_system* s, int op) {
  cudaError_t e = launch_unary(ctx(s), s->cur, s->k, s->b, s->n_host, op);
  if (e != cudaSuccess) return fail(s, SPH_ERR_CUDA, "unary launch: %s", cudaGetErrorString(e));
  if (op == SPH_OP_DRIFT) {
    s->cells_valid = false;
    s->lists_valid = false;
    s->hits_valid = false;
  }
  s->aux_fluid = s->aux_wall = false;
  return SPH_OK;
}

bool vector_field(int f) {
  return f == SPH_FIELD_X || f == SPH_FIELD_V || f == SPH_FIELD_A || f == SPH_FIELD_XSPH;
}

size_t field_bytes(int f, size_t n) {
  if (vector_field(f)) return 24 * n;
  if (f == SPH_FIELD_TYPE) return 4 * n;
  return 8 * n;
}



}  // namespace

namespace sphgpu {
LaunchCtx system_ctx(sph_system* s) { return ctx(s); }
int system_fail(sph_system* s, int code, const char* msg) { return fail(s, code, "%s", msg); }
}  // namespace sphgpu

extern "C" {

int sph_abi_version(void) { return SPHGPU_ABI_VERSION; }

const char* sph_last_error(const sph_system* s) { return s ? s->err.c_str() : "null handle"; }

// Validates the parameters and fills the host-side geometry and constants
// (no CUDA call).
static int setup_host(const sph_params* p, sph_system* s) {
  if (p->dim != 2 && p->dim != 3) return SPH_ERR_ARG;
  if (!(p->h > 0.0)) return SPH_ERR_ARG;  // structs.jl:59
  if (p->precision != SPH_PREC_FP64 && p->precision != SPH_PREC_MIXED) return SPH_ERR_ARG;
  if (p->vertical_axis < 0 || p->vertical_axis >= p->dim) return SPH_ERR_ARG;
  for (int d = 0; d < 3; ++d)
    if (!(p->domain_min[d] <= p->domain_max[d])) return SPH_ERR_ARG;
  if (p->dim == 2 && (p->domain_min[2] > 0.0 || p->domain_max[2] < 0.0)) return SPH_ERR_ARG;
  if (p->eos != SPH_EOS_TAIT && p->eos != SPH_EOS_LINEAR) return SPH_ERR_ARG;
  // the cell factor: the reference's cells (0 or 1) for every system, up to
  // 2 h for mixed-precision ones (the FP64 path sums in the reference's
  // neighbour order, which the cells define)
  const double cf = p->cell_factor == 0.0 ? 1.0 : p->cell_factor;
  if (!(cf >= 1.0 && cf <= 2.0)) return SPH_ERR_ARG;
  if (cf != 1.0 && p->precision != SPH_PREC_MIXED) return SPH_ERR_ARG;
  s->params = *p;
  // structs.jl:64-82, with cells of size Hc (H unless a mixed system asks
  // for larger ones)
  const double H = p->h;
  const double Hc = cf == 1.0 ? H : H * cf;
  // Mixed systems shift their grid by 5/16 of a cell.  A lattice whose
  // spacing divides the cell (h = 4 dr in 3D) otherwise has whole planes of
  // particles exactly on cell boundaries, which rounding in the first steps
  // scatters to either side: cells of 65 particles take three work items.
  // With the shift such planes lie a quarter spacing (h = 4 dr) or a tenth
  // (h = 4.8 dr) away from every boundary.  The pair set does not depend on
  // the grid; the FP64 path sums in the reference's cell order and keeps it.
  // Mixed systems also take the cell index from a product with 1/cell
  // (Consts.inv_cell); the key range below uses the same expression.
  double shift[3] = {0.0, 0.0, 0.0};
  const double inv_cell = p->precision == SPH_PREC_MIXED ? 1.0 / Hc : 0.0;
  const auto cell_coord = [&](double x, int d) {
    const double u = x - shift[d];
    return inv_cell != 0.0 ? u * inv_cell : u / Hc;
  };
  long long key_max = 1;
  for (int d = 0; d < 3; ++d) {
    shift[d] = p->precision == SPH_PREC_MIXED && d < p->dim ? Hc * (5.0 / 16.0) : 0.0;
    s->geo.key_phase[d] = (long long)std::floor(cell_coord(p->domain_min[d], d));
    s->geo.key_lim[d] =
        (long long)std::floor(cell_coord(p->domain_max[d], d)) - s->geo.key_phase[d] + 1;
    key_max *= s->geo.key_lim[d];
  }
  if (key_max <= 0 || key_max > 0x7fffffffLL - 8)
    return SPH_ERR_ARG;  // the cell table must be indexable with int32
  s->geo.key_max = (int)key_max;
  int nd = 0;
  const long long L0 = s->geo.key_lim[0], L1 = s->geo.key_lim[1];
  if (s->geo.key_lim[2] == 1) {
    for (int di = -1; di <= 1; ++di)
      for (int dj = -1; dj <= 1; ++dj) s->geo.key_diff[nd++] = (int)(di + L0 * dj);
  } else {
    for (int di = -1; di <= 1; ++di)
      for (int dj = -1; dj <= 1; ++dj)
        for (int dk = -1; dk <= 1; ++dk) s->geo.key_diff[nd++] = (int)(di + L0 * (dj + L1 * dk));
  }
  s->geo.n_diff = nd;
  // derived constants: same expressions as the CPU restatement
  Consts& k = s->k;
  k.dim = p->dim;
  k.warps = 4;
  k.split = 1;
  k.h = H;
  k.inv_h = 1.0 / H;
  const double h2 = H * H;
  if (p->dim == 2) {
    k.cw = 2.228169203286535 / h2;
    k.cr = -44.563384065730695 / (h2 * h2);
  } else {
    k.cw = 3.3422538049298023 / (h2 * H);
    k.cr = -66.84507609859604 / ((h2 * h2) * H);
  }
  k.mass = p->mass;
  k.rho0 = p->rho0;
  k.B = ((p->c0 * p->c0) * p->rho0) / 7.0;
  k.eos = p->eos;
  k.c2 = p->c0 * p->c0;
  k.rho0sq = p->rho0 * p->rho0;
  k.hdt = 0.5 * p->dt;
  k.dt = p->dt;
  k.eta2 = 0.01 * (p->h_smooth * p->h_smooth);
  k.alpha_c0 = p->alpha * p->c0;
  k.mcw = p->mass * k.cw;
  k.mcw5 = 5.0 * k.mcw;
  k.mcw4 = -4.0 * k.mcw;
  k.mcr = p->mass * k.cr;
  k.ca = -(k.alpha_c0 * p->h_smooth);
  k.h_smooth = p->h_smooth;
  k.eps_xsph = p->eps_xsph;
  k.gmag = std::fabs(p->gravity[p->vertical_axis]);
  k.col_height = p->col_height;
  k.vaxis = p->vertical_axis;
  for (int d = 0; d < 3; ++d) {
    k.g[d] = p->gravity[d];
    k.dmin[d] = p->domain_min[d];
    k.dmax[d] = p->domain_max[d];
  }
  const double band = 1.0 / 16384.0;  // 2^-14, see sph_pair64.cu
  k.cell = Hc;
  k.cellf = (float)Hc;
  for (int d = 0; d < 3; ++d) k.shift[d] = shift[d];
  k.inv_cell = inv_cell;
  k.s_lo = (float)(h2 * (1.0 - band));
  k.s_hi = (float)(h2 * (1.0 + band));
  // largest double whose correctly rounded square root is <= H
  double smax = h2;
  while (std::sqrt(smax) > H) smax = std::nextafter(smax, 0.0);
  while (std::sqrt(std::nextafter(smax, HUGE_VAL)) <= H) smax = std::nextafter(smax, HUGE_VAL);
  k.s_max = smax;
  // fixed-point positions X = x 2^fx_k with |X| < 2^62 inside the domain box
  // (particles outside it are removed by the binning)
  double span = 0.0;
  for (int d = 0; d < p->dim; ++d)
    span = std::max(span, std::max(std::fabs(p->domain_min[d]), std::fabs(p->domain_max[d])));
  int e = 0;
  std::frexp(span, &e);  // span < 2^e
  k.fx_k = std::max(-1000, std::min(1000, 62 - e));
  k.inv_hf = (float)k.inv_h;
  k.hf = (float)H;
  k.cwf = (float)k.cw;
  k.crf = (float)k.cr;
  k.massf = (float)k.mass;
  k.eta2f = (float)k.eta2;
  k.alpha_c0f = (float)k.alpha_c0;
  k.h_smoothf = (float)k.h_smooth;
  k.rho0f = (float)k.rho0;
  for (int d = 0; d < 3; ++d) k.gf[d] = (float)k.g[d];
  return SPH_OK;
}

// Bytes of the cell tables (fixed per system) and of the particle arena for
// capacity C.
static size_t cells_bytes(const sph_system* s) {
  const size_t nb = (size_t)s->geo.key_max + 3;
  const size_t scan_ints = scan_tmp_ints((int)nb) + 64;
  return align_up(4 * nb) * 5 + align_up(4 * scan_ints) + 2048;
}

int sph_create(const sph_params* p, int device, sph_system** out) {
  if (!p || !out) return SPH_ERR_ARG;
  *out = nullptr;
  sph_system* s = new sph_system();
  const int rc = setup_host(p, s);
  if (rc) {
    delete s;
    return rc;
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) {
    cudaGetLastError();
    delete s;
    return SPH_ERR_CUDA;
  }
  s->device = device;
  DeviceGuard guard(device);
  if (cudaDeviceGetAttribute(&s->sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess ||
      s->sms < 1) {
    cudaGetLastError();
    s->sms = 1;
  }
  if (cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess) {
    cudaGetLastError();
    delete s;
    return SPH_ERR_CUDA;
  }
  if (p->precision == SPH_PREC_FP64) {
    // the word the FP64 passes report a row shortfall in: host memory the
    // device writes directly, so the host reads it without a copy
    void* dev_alias = nullptr;
    if (cudaHostAlloc((void**)&s->need_host, sizeof(unsigned long long), cudaHostAllocMapped) !=
            cudaSuccess ||
        cudaHostGetDevicePointer(&dev_alias, s->need_host, 0) != cudaSuccess) {
      cudaGetLastError();
      if (s->need_host) cudaFreeHost(s->need_host);
      cudaStreamDestroy(s->stream);
      delete s;
      return SPH_ERR_CUDA;
    }
    *s->need_host = 0;
    s->b.need_host = (unsigned long long*)dev_alias;
  }
  const size_t nb = (size_t)s->geo.key_max + 3;
  const size_t scan_ints = scan_tmp_ints((int)nb) + 64;
  const size_t bytes = cells_bytes(s);
  void* cells = nullptr;
  if (cudaMalloc(&cells, bytes) != cudaSuccess) {
    cudaGetLastError();
    if (s->need_host) cudaFreeHost(s->need_host);
    cudaStreamDestroy(s->stream);
    delete s;
    return SPH_ERR_NOMEM;
  }
  s->cells = cells;
  char* c = (char*)cells;
  s->b.counts = (int*)c;
  c += align_up(4 * nb);
  s->b.cell_start = (int*)c;
  c += align_up(4 * nb);
  s->b.item_off = (int*)c;
  c += align_up(4 * nb);
  s->b.cell_fluid = (int*)c;
  c += align_up(4 * nb);
  s->b.chunk_off = (int*)c;
  c += align_up(4 * nb);
  s->b.scan_tmp = (int*)c;
  c += align_up(4 * scan_ints);
  s->b.d_n = (int*)c;
  s->b.d_nrem = (int*)(c + 256);
  s->b.d_err = (int*)(c + 512);
  s->b.d_pairs = (unsigned long long*)(c + 768);
  s->b.d_cat = (unsigned long long*)(c + 1024);
  s->b.d_npairs = (unsigned long long*)(c + 1280);
  s->b.d_pover = (int*)(c + 1288);
  s->b.d_rover = (int*)(c + 1292);
  s->b.d_rowsum = (unsigned long long*)(c + 1296);
  s->b.d_nwall = (int*)(c + 1304);
  s->d_debug = (int*)(c + 1536);
  s->b.work_ctr = (int*)(c + 1600);
  if (cudaMemsetAsync(cells, 0, bytes, s->stream) != cudaSuccess ||
      cudaStreamSynchronize(s->stream) != cudaSuccess) {
    cudaGetLastError();
    cudaFree(cells);
    if (s->need_host) cudaFreeHost(s->need_host);
    cudaStreamDestroy(s->stream);
    delete s;
    return SPH_ERR_CUDA;
  }
  *out = s;
  return SPH_OK;
}

int sph_destroy(sph_system* s) {
  if (!s) return SPH_ERR_ARG;
  DeviceGuard guard(s->device);
  if (s->solo) sph_batch_destroy(s->solo);
  cudaStreamSynchronize(s->stream);
  for (auto& p : s->pending) {
    cudaEventDestroy(p.start);
    cudaEventDestroy(p.stop);
  }
  for (auto e : s->pool) cudaEventDestroy(e);
  if (s->open_start) cudaEventDestroy(s->open_start);
  if (s->arena) cudaFree(s->arena);
  if (s->rowbuf) cudaFree(s->rowbuf);
  if (s->need_host) cudaFreeHost(s->need_host);
  if (s->cells) cudaFree(s->cells);
  if (s->query) cudaFree(s->query);
  for (auto e : s->io_ev)
    if (e) cudaEventDestroy(e);
  if (s->io_stream) cudaStreamDestroy(s->io_stream);
  cudaStreamDestroy(s->stream);
  delete s;
  return SPH_OK;
}

int sph_geometry(const sph_system* s, int64_t key_phase[3], int64_t key_lim[3], int64_t* key_max,
                 int64_t key_diff[27], int32_t* n_diff) {
  if (!s || !key_phase || !key_lim || !key_max || !key_diff || !n_diff) return SPH_ERR_ARG;
  for (int d = 0; d < 3; ++d) {
    key_phase[d] = s->geo.key_phase[d];
    key_lim[d] = s->geo.key_lim[d];
  }
  *key_max = s->geo.key_max;
  for (int i = 0; i < s->geo.n_diff; ++i) key_diff[i] = s->geo.key_diff[i];
  *n_diff = s->geo.n_diff;
  return SPH_OK;
}

int sph_upload(sph_system* s, int64_t n, const double* x, const double* v, const double* rho,
               const double* rho_ref, const int32_t* type) {
  if (!s) return SPH_ERR_ARG;
  // the pair passes pack a particle index into 27 bits of a queue entry
  if (n < 0 || n >= (1LL << 27)) return fail(s, SPH_ERR_ARG, "invalid particle count %lld (limit 2^27 - 1)", (long long)n);
  if (n > 0 && !x) return fail(s, SPH_ERR_ARG, "x is null");
  if (s->params.dim == 2) {
    for (int64_t i = 0; i < n; ++i)
      if (x[3 * i + 2] != 0.0 || (v && v[3 * i + 2] != 0.0))
        return fail(s, SPH_ERR_ARG, "2D system: particle %lld has a nonzero z component", (long long)i);
  }
  if (type)
    for (int64_t i = 0; i < n; ++i)
      if (type[i] != SPH_FLUID && type[i] != SPH_WALL)
        return fail(s, SPH_ERR_ARG, "particle %lld has unknown type %d", (long long)i, type[i]);
  DeviceGuard guard(s->device);
  int rc = ensure_capacity(s, (int)n);
  if (rc) return rc;
  char* st = (char*)s->staging;
  const size_t N = (size_t)n;
  double* dx = (double*)st;
  double* dv = (double*)(st + 24 * N);
  double* drho = (double*)(st + 48 * N);
  double* drr = (double*)(st + 56 * N);
  int* dtype = (int*)(st + 64 * N);
  if (n > 0) {
    CK(cudaMemcpyAsync(dx, x, 24 * N, cudaMemcpyHostToDevice, s->stream));
    if (v) CK(cudaMemcpyAsync(dv, v, 24 * N, cudaMemcpyHostToDevice, s->stream));
    if (rho) CK(cudaMemcpyAsync(drho, rho, 8 * N, cudaMemcpyHostToDevice, s->stream));
    if (rho_ref) CK(cudaMemcpyAsync(drr, rho_ref, 8 * N, cudaMemcpyHostToDevice, s->stream));
    if (type) CK(cudaMemcpyAsync(dtype, type, 4 * N, cudaMemcpyHostToDevice, s->stream));
  }
  cudaError_t e = launch_upload(ctx(s), s->cur, s->k, s->b, (int)n, dx, v ? dv : nullptr,
                                rho ? drho : nullptr, rho_ref ? drr : nullptr,
                                type ? dtype : nullptr);
  if (e != cudaSuccess) return fail(s, SPH_ERR_CUDA, "upload: %s", cudaGetErrorString(e));
  CK(cudaStreamSynchronize(s->stream));
  s->n_host = (int)n;
  // a captured step sized its grids by the previous count: capture again
  ++s->generation;
  s->cells_valid = false;
  s->aux_fluid = s->aux_wall = false;
  s->lists_valid = false;
  s->hits_valid = false;
  return SPH_OK;
}

// Counts (and, when `write`, generates into x / type at the running offset)
// the particles of every shape on `stream`; temporaries are allocated here.
static int shapes_run(int dim, const sph_shape* shapes, int count, cudaStream_t stream,
                      const LaunchCtx* c, double* x, int* type, long long* total_out,
                      std::string* err) {
  std::vector<LatticeShape> ls(count);
  std::vector<std::vector<double>> offs(count);
  long long maxp = 0, maxo = 0;
  for (int i = 0; i < count; ++i) {
    if (lattice_prepare(shapes[i], dim, ls[i], offs[i]) != SPH_OK) {
      if (err) *err = "invalid shape " + std::to_string(i);
      return SPH_ERR_ARG;
    }
    const long long np = lattice_points(ls[i]);
    if (np > 0x7fffffffLL - 4096) {
      if (err) *err = "shape " + std::to_string(i) + ": bounding box holds more than 2^31 points";
      return SPH_ERR_ARG;
    }
    maxp = std::max(maxp, np);
    maxo = std::max(maxo, (long long)offs[i].size());
  }
  const size_t scan_ints = scan_tmp_ints((int)(maxp + 1)) + 64;
  const size_t bytes = 8 * (size_t)(maxp + 1) + 4 * scan_ints + 8 * (size_t)(maxo + 3) + 1024;
  void* tmp = nullptr;
  if (cudaMalloc(&tmp, bytes) != cudaSuccess) {
    cudaGetLastError();
    if (err) *err = "cannot allocate the generation scratch";
    return SPH_ERR_NOMEM;
  }
  char* p = (char*)tmp;
  int* flags = (int*)p;
  int* pos = flags + (maxp + 1);
  int* stmp = pos + (maxp + 1);
  double* doffs = (double*)(((uintptr_t)(stmp + scan_ints) + 255) & ~(uintptr_t)255);
  LaunchCtx lc = c ? *c : LaunchCtx{stream, nullptr, nullptr};
  long long total = 0;
  int rc = SPH_OK;
  for (int i = 0; i < count && rc == SPH_OK; ++i) {
    const long long np = lattice_points(ls[i]);
    if (!offs[i].empty() &&
        cudaMemcpyAsync(doffs, offs[i].data(), 8 * offs[i].size(), cudaMemcpyHostToDevice,
                        stream) != cudaSuccess) {
      rc = SPH_ERR_CUDA;
      break;
    }
    // flags[np] = 0 so that pos[np] is the shape's count
    if (cudaMemsetAsync(flags + np, 0, sizeof(int), stream) != cudaSuccess ||
        launch_lattice_flags(lc, ls[i], doffs, flags) != cudaSuccess ||
        launch_scan(lc, flags, pos, (int)(np + 1), stmp) != cudaSuccess) {
      rc = SPH_ERR_CUDA;
      break;
    }
    int cnt = 0;
    if (cudaMemcpyAsync(&cnt, pos + np, sizeof(int), cudaMemcpyDeviceToHost, stream) !=
            cudaSuccess ||
        cudaStreamSynchronize(stream) != cudaSuccess) {
      rc = SPH_ERR_CUDA;
      break;
    }
    if (x && launch_lattice_write(lc, ls[i], flags, pos, x, type, (int)total) != cudaSuccess) {
      rc = SPH_ERR_CUDA;
      break;
    }
    total += cnt;
  }
  if (rc == SPH_OK && cudaStreamSynchronize(stream) != cudaSuccess) rc = SPH_ERR_CUDA;
  if (rc != SPH_OK) {
    cudaGetLastError();
    if (err) *err = "particle generation failed";
  }
  cudaFree(tmp);
  *total_out = total;
  return rc;
}

// The temporary device bytes shapes_run allocates for these shapes (host
// arithmetic only; the same expressions as shapes_run).
static int shapes_scratch(int dim, const sph_shape* shapes, int count, size_t* out) {
  long long maxp = 0, maxo = 0;
  for (int i = 0; i < count; ++i) {
    LatticeShape ls;
    std::vector<double> offs;
    if (lattice_prepare(shapes[i], dim, ls, offs) != SPH_OK) return SPH_ERR_ARG;
    const long long np = lattice_points(ls);
    if (np > 0x7fffffffLL - 4096) return SPH_ERR_ARG;
    maxp = std::max(maxp, np);
    maxo = std::max(maxo, (long long)offs.size());
  }
  const size_t scan_ints = scan_tmp_ints((int)(maxp + 1)) + 64;
  *out = 8 * (size_t)(maxp + 1) + 4 * scan_ints + 8 * (size_t)(maxo + 3) + 1024;
  return SPH_OK;
}

int sph_generate_scratch(int dim, const sph_shape* shapes, int count, uint64_t* bytes) {
  if (!bytes || count < 0 || (count > 0 && !shapes) || (dim != 2 && dim != 3)) return SPH_ERR_ARG;
  size_t b = 0;
  const int rc = shapes_scratch(dim, shapes, count, &b);
  if (rc == SPH_OK) *bytes = (uint64_t)b;
  return rc;
}

int sph_device_memory(int device, uint64_t* free_bytes, uint64_t* total_bytes) {
  if (!free_bytes || !total_bytes) return SPH_ERR_ARG;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) {
    cudaGetLastError();
    return SPH_ERR_CUDA;
  }
  DeviceGuard guard(device);
  size_t f = 0, t = 0;
  if (cudaMemGetInfo(&f, &t) != cudaSuccess) {
    cudaGetLastError();
    return SPH_ERR_CUDA;
  }
  *free_bytes = (uint64_t)f;
  *total_bytes = (uint64_t)t;
  return SPH_OK;
}

int sph_shape_count(int device, int dim, const sph_shape* shapes, int count, int64_t* n_out) {
  if (!n_out || count < 0 || (count > 0 && !shapes) || (dim != 2 && dim != 3)) return SPH_ERR_ARG;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) {
    cudaGetLastError();
    return SPH_ERR_CUDA;
  }
  DeviceGuard guard(device);
  cudaStream_t st = nullptr;
  if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) {
    cudaGetLastError();
    return SPH_ERR_CUDA;
  }
  long long total = 0;
  const int rc = shapes_run(dim, shapes, count, st, nullptr, nullptr, nullptr, &total, nullptr);
  cudaStreamDestroy(st);
  if (rc == SPH_OK) *n_out = total;
  return rc;
}

int sph_generate(sph_system* s, const sph_shape* shapes, int count, int64_t* n_out) {
  if (!s || count < 0 || (count > 0 && !shapes)) return SPH_ERR_ARG;
  DeviceGuard guard(s->device);
  long long total = 0;
  std::string err;
  int rc = shapes_run(s->params.dim, shapes, count, s->stream, nullptr, nullptr, nullptr, &total,
                      &err);
  if (rc) return fail(s, rc, "%s", err.c_str());
  // the pair passes pack a particle index into 27 bits of a list entry
  if (total >= (1LL << 27))
    return fail(s, SPH_ERR_ARG, "%lld particles exceed the limit 2^27 - 1", total);
  rc = ensure_capacity(s, (int)total);
  if (rc) return rc;
  const size_t N = (size_t)total;
  double* dx = (double*)s->staging;
  int* dtype = (int*)((char*)s->staging + 64 * N);
  long long again = 0;
  const LaunchCtx c = ctx(s);
  rc = shapes_run(s->params.dim, shapes, count, s->stream, &c, dx, dtype, &again, &err);
  if (rc) return fail(s, rc, "%s", err.c_str());
  cudaError_t e = launch_upload(ctx(s), s->cur, s->k, s->b, (int)total, dx, nullptr, nullptr,
                                nullptr, dtype);
  if (e != cudaSuccess) return fail(s, SPH_ERR_CUDA, "generate: %s", cudaGetErrorString(e));
  CK(cudaStreamSynchronize(s->stream));
  s->n_host = (int)total;
  ++s->generation;  // as in sph_upload
  s->cells_valid = false;
  s->aux_fluid = s->aux_wall = false;
  s->lists_valid = false;
  s->hits_valid = false;
  if (n_out) *n_out = total;
  return SPH_OK;
}

int sph_num_particles(sph_system* s, int64_t* n) {
  if (!s || !n) return SPH_ERR_ARG;
  DeviceGuard guard(s->device);
  int c = 0;
  int rc = read_count(s, &c);
  if (rc) return rc;
  *n = c;
  return SPH_OK;
}

int sph_get_field(sph_system* s, int field, void* out) {
  if (!s || !out) return SPH_ERR_ARG;
  if (field < SPH_FIELD_X || field > SPH_FIELD_KEY) return fail(s, SPH_ERR_ARG, "unknown field %d", field);
  DeviceGuard guard(s->device);
  int n = 0;
  int rc = read_count(s, &n);
  if (rc) return rc;
  if (n == 0) return SPH_OK;
  cudaError_t e = launch_field(ctx(s), s->cur, s->k, s->b, s->n_host, field, 0, s->staging);
  if (e != cudaSuccess) return fail(s, SPH_ERR_CUDA, "field: %s", cudaGetErrorString(e));
  CK(cudaMemcpyAsync(out, s->staging, field_bytes(field, n), cudaMemcpyDeviceToHost, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  return SPH_OK;
}

// The host-side checks of a field about to be set (2D systems: no z
// component; types: fluid or wall only).
static int check_set(sph_system* s, int field, const void* in, int n) {
  if (s->params.dim == 2 && (field == SPH_FIELD_X || field == SPH_FIELD_V)) {
    const double* v = (const double*)in;
    for (int i = 0; i < n; ++i)
      if (v[3 * i + 2] != 0.0)
        return fail(s, SPH_ERR_ARG, "2D system: particle %d has a nonzero z component", i);
  }
  if (field == SPH_FIELD_TYPE) {
    const int32_t* t = (const int32_t*)in;
    for (int i = 0; i < n; ++i)
      if (t[i] != SPH_FLUID && t[i] != SPH_WALL)
        return fail(s, SPH_ERR_ARG, "particle %d has unknown type %d", i, t[i]);
  }
  return SPH_OK;
}

// What setting a field invalidates.
static void after_set(sph_system* s, int field) {
  if (field == SPH_FIELD_X) s->cells_valid = false;
  if (field == SPH_FIELD_X || field == SPH_FIELD_TYPE) s->lists_valid = s->hits_valid = false;
  s->aux_fluid = s->aux_wall = false;
}

int sph_set_field(sph_system* s, int field, const void* in) {
  if (!s || !in) return SPH_ERR_ARG;
  if (field < SPH_FIELD_X || field > SPH_FIELD_TYPE)
    return fail(s, SPH_ERR_ARG, "field %d cannot be set", field);
  DeviceGuard guard(s->device);
  int n = 0;
  int rc = read_count(s, &n);
  if (rc) return rc;
  if (n == 0) return SPH_OK;
  rc = check_set(s, field, in, n);
  if (rc) return rc;
  CK(cudaMemcpyAsync(s->staging, in, field_bytes(field, n), cudaMemcpyHostToDevice, s->stream));
  cudaError_t e = launch_field(ctx(s), s->cur, s->k, s->b, s->n_host, field, 1, s->staging);
  if (e != cudaSuccess) return fail(s, SPH_ERR_CUDA, "field: %s", cudaGetErrorString(e));
  CK(cudaStreamSynchronize(s->stream));
  after_set(s, field);
  return SPH_OK;
}

int sph_create_cell_list(sph_system* s) {
  if (!s) return SPH_ERR_ARG;
  DeviceGuard guard(s->device);
  return binning(s, 0, kGatherAll);
}

int sph_apply(sph_system* s, int op, int self) {
  if (!s) return SPH_ERR_ARG;
  if (op != SPH_OP_DENSITY && op != SPH_OP_DENSITY_REF && op != SPH_OP_FORCE &&
      op != SPH_OP_WALL_PRESSURE) {
    if (op >= SPH_OP_RESET_RHO && op <= SPH_OP_HYDROSTATIC) return sph_apply_unary(s, op);
    return fail(s, SPH_ERR_ARG, "unknown operator %d", op);
  }
  if (!s->cells_valid)
    return fail(s, SPH_ERR_STATE, "positions changed since create_cell_list!; call it first");
  DeviceGuard guard(s->device);
  return pair_pass(s, op, self ? 1 : 0, 0, 0);
}

int sph_apply_unary(sph_system* s, int op) {
  if (!s) return SPH_ERR_ARG;
  if (op < SPH_OP_RESET_RHO || op > SPH_OP_HYDROSTATIC)
    return fail(s, SPH_ERR_ARG, "unknown unary operator %d", op);
  DeviceGuard guard(s->device);
  return unary(s, op);
}

static int sum_common(sph_system* s, int func, int64_t nq, const double* x, const int64_t* idx,
                      double* out) {
  if (!s || (nq > 0 && !out) || nq < 0) return SPH_ERR_ARG;
  if (func < SPH_SUM_DENSITY || func > SPH_SUM_SHEPARD) return fail(s, SPH_ERR_ARG, "unknown sum function %d", func);
  if (!s->cells_valid) return fail(s, SPH_ERR_STATE, "cell list is stale; call create_cell_list! first");
  if (nq == 0) return SPH_OK;
  if (nq > 0x7fffffffLL / 4) return fail(s, SPH_ERR_ARG, "too many query points");
  DeviceGuard guard(s->device);
  int n = 0;
  if (idx) {
    int rc = read_count(s, &n);
    if (rc) return rc;
    for (int64_t i = 0; i < nq; ++i)
      if (idx[i] < 0 || idx[i] >= n) return fail(s, SPH_ERR_ARG, "particle index %lld out of range", (long long)idx[i]);
  }
  const size_t need = (size_t)nq * 32;
  if (need > s->query_bytes) {
    if (s->query) CK(cudaFree(s->query));
    s->query = nullptr;
    s->query_bytes = 0;
    if (cudaMalloc(&s->query, need) != cudaSuccess) {
      cudaGetLastError();
      return fail(s, SPH_ERR_NOMEM, "cannot allocate the query buffer");
    }
    s->query_bytes = need;
  }
  double* dq = s->query;                         // nq x 3 points or nq indices
  double* dout = s->query + 3 * (size_t)nq;      // nq results
  if (idx)
    CK(cudaMemcpyAsync(dq, idx, 8 * (size_t)nq, cudaMemcpyHostToDevice, s->stream));
  else
    CK(cudaMemcpyAsync(dq, x, 24 * (size_t)nq, cudaMemcpyHostToDevice, s->stream));
  cudaError_t e = launch_sum(ctx(s), s->cur, s->geo, s->k, s->b, func, (int)nq,
                             idx ? nullptr : dq, idx ? (const long long*)dq : nullptr, dout);
  if (e != cudaSuccess) return fail(s, SPH_ERR_CUDA, "sum: %s", cudaGetErrorString(e));
  CK(cudaMemcpyAsync(out, dout, 8 * (size_t)nq, cudaMemcpyDeviceToHost, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  return SPH_OK;
}

int sph_sum_point(sph_system* s, int func, int64_t nq, const double* x, double* out) {
  if (nq > 0 && !x) return SPH_ERR_ARG;
  return sum_common(s, func, nq, x, nullptr, out);
}

int sph_sum_particle(sph_system* s, int func, int64_t nq, const int64_t* index, double* out) {
  if (nq > 0 && !index) return SPH_ERR_ARG;
  return sum_common(s, func, nq, nullptr, index, out);
}

// one verlet_step!: every launch is asynchronous on the handle's stream (no
// host synchronisation), so the sequence can be captured into a CUDA graph
static int step_once(sph_system* s) {
  int rc = binning(s, 1, kGatherStep);  // kick + drift + create_cell_list!
  if (rc) return rc;
  rc = pair_pass(s, SPH_OP_DENSITY, 1, 1, 1);  // reset_rho!, find_rho!(self), EOS
  if (rc) return rc;
  rc = pair_pass(s, SPH_OP_WALL_PRESSURE, 0, 0, 0);
  if (rc) return rc;
  rc = pair_pass(s, SPH_OP_FORCE, 0, 1, 0);  // reset_a!, internal_force!
  if (rc) return rc;
  return unary(s, SPH_OP_KICK);
}

// Steps per call from which sph_step replays a captured CUDA graph.
constexpr int kGraphSteps = 4;

int sph_step(sph_system* s, int nsteps) {
  if (!s || nsteps < 0) return SPH_ERR_ARG;
  DeviceGuard guard(s->device);
  // Many steps at once, without per-kernel timing: replay a captured
  // two-step CUDA graph of this system alone (a batch of one, kept until the
  // system's buffers, count or tuning change) instead of launching every
  // kernel from the host -- small systems are bound by those launches.  The
  // graph holds the kernels of step_once, so the results are the same.
  if (nsteps >= kGraphSteps && !s->profiling && s->n_host > 0 && s->arena) {
    if (!s->solo) {
      sph_system* self = s;
      const int rc = sph_batch_create(&self, 1, &s->solo);
      if (rc) return fail(s, rc, "cannot set up the step graph");
    }
    sph_batch* b = s->solo;
    if (b->fused_warps != s->k.warps) sph_batch_set_tuning(b, s->k.warps);
    if (b->exec && (nsteps & 1) && b->cur0[0] != s->cur.x[0]) {
      // an odd count on the other ping-pong half than the graph's: the
      // single step first brings it back, and the graph serves the rest
      const int rc = step_once(s);
      if (rc) return rc;
      --nsteps;
    }
    const long long l0 = b->launches;
    const int rc = sph_batch_step(b, nsteps);
    s->total_launches += b->launches - l0;
    if (rc) return fail(s, rc, "step graph: %s", b->err.c_str());
    return SPH_OK;
  }
  for (int it = 0; it < nsteps; ++it) {
    const int rc = step_once(s);
    if (rc) return rc;
  }
  return SPH_OK;
}

// The phase of a step after which a field read by sph_step_io is final:
// 0 after the binning (kick and drift done, state sorted), 1 after the wall
// pressure (density and pressure of every particle), 2 at the end (the
// force pass and the closing kick).
static int final_phase(int field) {
  switch (field) {
    case SPH_FIELD_RHO:
    case SPH_FIELD_P: return 1;
    case SPH_FIELD_V:
    case SPH_FIELD_A:
    case SPH_FIELD_XSPH: return 2;
    default: return 0;
  }
}

int sph_step_io(sph_system* s, int nin, const int32_t* in_fields, const void* const* in, int nout,
                const int32_t* out_fields, void* const* out) {
  if (!s || nin < 0 || nout < 0 || (nin > 0 && (!in_fields || !in)) ||
      (nout > 0 && (!out_fields || !out)))
    return SPH_ERR_ARG;
  for (int i = 0; i < nin; ++i)
    if (in_fields[i] < SPH_FIELD_X || in_fields[i] > SPH_FIELD_TYPE || !in[i])
      return fail(s, SPH_ERR_ARG, "input %d: field %d cannot be set", i, in_fields[i]);
  for (int i = 0; i < nout; ++i)
    if (out_fields[i] < SPH_FIELD_X || out_fields[i] > SPH_FIELD_KEY || !out[i])
      return fail(s, SPH_ERR_ARG, "output %d: unknown field %d", i, out_fields[i]);
  DeviceGuard guard(s->device);
  int n = 0;
  int rc = read_count(s, &n);
  if (rc) return rc;
  if (n == 0) return sph_step(s, 1);
  if (!s->io_stream) {
    CK(cudaStreamCreateWithFlags(&s->io_stream, cudaStreamNonBlocking));
    for (auto& e : s->io_ev) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  }
  // the inputs, one after the other through the staging area
  for (int i = 0; i < nin; ++i) {
    rc = check_set(s, in_fields[i], in[i], n);
    if (rc) return rc;
    CK(cudaMemcpyAsync(s->staging, in[i], field_bytes(in_fields[i], n), cudaMemcpyHostToDevice,
                       s->stream));
    cudaError_t e =
        launch_field(ctx(s), s->cur, s->k, s->b, s->n_host, in_fields[i], 1, s->staging);
    if (e != cudaSuccess) return fail(s, SPH_ERR_CUDA, "field: %s", cudaGetErrorString(e));
    after_set(s, in_fields[i]);
  }
  // step_once, with an event after each phase that makes outputs final
  rc = binning(s, 1, kGatherStep);
  if (rc) return rc;
  CK(cudaEventRecord(s->io_ev[0], s->stream));
  // the particle count after the binning's removals sizes the reads
  rc = read_count(s, &n);
  if (rc) return rc;
  rc = pair_pass(s, SPH_OP_DENSITY, 1, 1, 1);
  if (!rc) rc = pair_pass(s, SPH_OP_WALL_PRESSURE, 0, 0, 0);
  if (rc) return rc;
  CK(cudaEventRecord(s->io_ev[1], s->stream));
  // the reads final so far start now, on the second stream, while the rest
  // of the step runs; each phase's fields share the staging area, which the
  // next phase reuses once that stream has copied them out.  A copy into
  // pageable memory would hold the host until it is done, so then every
  // read waits for the end of the step.
  bool pinned = true;
  for (int i = 0; i < nout && pinned; ++i) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, out[i]) != cudaSuccess) {
      cudaGetLastError();
      pinned = false;
    } else {
      pinned = a.type == cudaMemoryTypeHost;
    }
  }
  const LaunchCtx quiet{s->io_stream, nullptr, nullptr};
  const State cur = s->cur;  // the sorted state of this step
  const size_t stage = 72 * (size_t)s->cap + 512;  // the staging area's bytes
  auto reads = [&](int phase) -> int {
    CK(cudaStreamWaitEvent(s->io_stream, s->io_ev[phase], 0));
    size_t off = 0;
    for (int i = 0; i < nout; ++i) {
      if ((pinned ? final_phase(out_fields[i]) : 2) != phase) continue;
      const size_t bytes = field_bytes(out_fields[i], n);
      if (off + bytes > stage) {  // the area is full: let the copies drain
        CK(cudaStreamSynchronize(s->io_stream));
        off = 0;
      }
      char* st = (char*)s->staging + off;
      cudaError_t e = launch_field(quiet, cur, s->k, s->b, s->n_host, out_fields[i], 0, st);
      if (e != cudaSuccess) return fail(s, SPH_ERR_CUDA, "field: %s", cudaGetErrorString(e));
      CK(cudaMemcpyAsync(out[i], st, bytes, cudaMemcpyDeviceToHost, s->io_stream));
      off += align_up(bytes);
    }
    return SPH_OK;
  };
  rc = reads(0);
  if (!rc) rc = reads(1);
  if (rc) return rc;
  rc = pair_pass(s, SPH_OP_FORCE, 0, 1, 0);
  if (!rc) rc = unary(s, SPH_OP_KICK);
  if (rc) return rc;
  CK(cudaEventRecord(s->io_ev[2], s->stream));
  rc = reads(2);
  if (rc) return rc;
  CK(cudaStreamSynchronize(s->io_stream));
  CK(cudaStreamSynchronize(s->stream));
  return SPH_OK;
}

int sph_init_state(sph_system* s) {
  if (!s) return SPH_ERR_ARG;
  DeviceGuard guard(s->device);
  int rc = binning(s, 0, kGatherAll);
  if (!rc) rc = unary(s, SPH_OP_RESET_RHO_REF);
  if (!rc) rc = pair_pass(s, SPH_OP_DENSITY_REF, 1, 0, 0);
  if (!rc) rc = unary(s, SPH_OP_HYDROSTATIC);
  if (!rc) rc = unary(s, SPH_OP_RESET_RHO);
  if (!rc) rc = pair_pass(s, SPH_OP_DENSITY, 1, 0, 0);
  if (!rc) rc = unary(s, SPH_OP_EOS);
  if (!rc) rc = pair_pass(s, SPH_OP_WALL_PRESSURE, 0, 0, 0);
  if (!rc) rc = unary(s, SPH_OP_RESET_A);
  if (!rc) rc = pair_pass(s, SPH_OP_FORCE, 0, 0, 0);
  return rc;
}

int sph_pair_count(sph_system* s, uint64_t* pairs, int reset) {
  if (!s || !pairs) return SPH_ERR_ARG;
  DeviceGuard guard(s->device);
  unsigned long long v = 0;
  CK(cudaMemcpyAsync(&v, s->b.d_pairs, sizeof v, cudaMemcpyDeviceToHost, s->stream));
  if (reset) CK(cudaMemsetAsync(s->b.d_pairs, 0, sizeof v, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  *pairs = v;
  return SPH_OK;
}

int sph_pair_stats(sph_system* s, uint64_t counts[8], int reset) {
  if (!s || !counts) return SPH_ERR_ARG;
  DeviceGuard guard(s->device);
  unsigned long long v[kNumCat];
  CK(cudaMemcpyAsync(v, s->b.d_cat, sizeof v, cudaMemcpyDeviceToHost, s->stream));
  if (reset) CK(cudaMemsetAsync(s->b.d_cat, 0, sizeof v, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  for (int i = 0; i < kNumCat; ++i) counts[i] = v[i];
  return SPH_OK;
}

int sph_synchronize(sph_system* s) {
  if (!s) return SPH_ERR_ARG;
  DeviceGuard guard(s->device);
  CK(cudaStreamSynchronize(s->stream));
  int errbits = 0;
  CK(cudaMemcpyAsync(&errbits, s->b.d_err, sizeof(int), cudaMemcpyDeviceToHost, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  if (errbits) {
    CK(cudaMemsetAsync(s->b.d_err, 0, sizeof(int), s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return fail(s, SPH_ERR_DEVICE, "device error bits 0x%x", errbits);
  }
  return SPH_OK;
}

int sph_stream(sph_system* s, void** stream) {
  if (!s || !stream) return SPH_ERR_ARG;
  *stream = (void*)s->stream;
  return SPH_OK;
}

int sph_debug_pairs(sph_system* s, int64_t* pairs, int64_t cap, int64_t* count) {
  if (!s || !count || cap < 0 || (cap > 0 && !pairs)) return SPH_ERR_ARG;
  if (!s->cells_valid) return fail(s, SPH_ERR_STATE, "cell list is stale; call create_cell_list! first");
  DeviceGuard guard(s->device);
  int n = 0;
  int rc = read_count(s, &n);
  if (rc) return rc;
  *count = 0;
  if (n == 0) return SPH_OK;
  int* dcounts = (int*)s->staging;
  long long* doff = (long long*)((char*)s->staging + align_up(4 * (size_t)n));
  cudaError_t e = launch_debug_pairs(ctx(s), s->cur, s->geo, s->k, s->b, s->n_host, 0, dcounts,
                                     nullptr, nullptr, 0);
  if (e != cudaSuccess) return fail(s, SPH_ERR_CUDA, "pairs: %s", cudaGetErrorString(e));
  std::vector<int> hc(n);
  std::vector<long long> ho(n);
  CK(cudaMemcpyAsync(hc.data(), dcounts, 4 * (size_t)n, cudaMemcpyDeviceToHost, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  long long total = 0;
  for (int i = 0; i < n; ++i) {
    ho[i] = total;
    total += hc[i];
  }
  *count = total;
  if (cap == 0) return SPH_OK;
  CK(cudaMemcpyAsync(doff, ho.data(), 8 * (size_t)n, cudaMemcpyHostToDevice, s->stream));
  const long long m = total < cap ? total : cap;
  long long* dpairs = nullptr;
  if (cudaMalloc(&dpairs, 16 * (size_t)(m > 0 ? m : 1)) != cudaSuccess) {
    cudaGetLastError();
    return fail(s, SPH_ERR_NOMEM, "cannot allocate the pair list");
  }
  e = launch_debug_pairs(ctx(s), s->cur, s->geo, s->k, s->b, s->n_host, 1, dcounts, doff, dpairs, m);
  cudaError_t e2 = cudaMemcpyAsync(pairs, dpairs, 16 * (size_t)m, cudaMemcpyDeviceToHost, s->stream);
  cudaError_t e3 = cudaStreamSynchronize(s->stream);
  cudaFree(dpairs);
  if (e != cudaSuccess || e2 != cudaSuccess || e3 != cudaSuccess)
    return fail(s, SPH_ERR_CUDA, "pair list transfer failed");
  return SPH_OK;
}

int sph_debug_hits(sph_system* s, int64_t* pairs, int64_t cap, int64_t* count) {
  if (!s || !count || cap < 0 || (cap > 0 && !pairs)) return SPH_ERR_ARG;
  if (!s->cells_valid || !s->hits_valid)
    return fail(s, SPH_ERR_STATE, "no density pass since the last create_cell_list!");
  DeviceGuard guard(s->device);
  int n = 0;
  int rc = read_count(s, &n);
  if (rc) return rc;
  *count = 0;
  if (n == 0) return SPH_OK;
  const int mixed = s->params.precision == SPH_PREC_MIXED ? 1 : 0;
  int* dcounts = (int*)s->staging;
  long long* doff = (long long*)((char*)s->staging + align_up(4 * (size_t)n));
  CK(cudaMemsetAsync(s->d_debug, 0, sizeof(int), s->stream));
  cudaError_t e = launch_debug_hits(ctx(s), s->cur, s->geo, s->b, s->n_host, mixed, 0, dcounts,
                                    nullptr, nullptr, 0, s->d_debug);
  if (e != cudaSuccess) return fail(s, SPH_ERR_CUDA, "hits: %s", cudaGetErrorString(e));
  std::vector<int> hc(n);
  std::vector<long long> ho(n);
  int bad = 0;
  CK(cudaMemcpyAsync(hc.data(), dcounts, 4 * (size_t)n, cudaMemcpyDeviceToHost, s->stream));
  CK(cudaMemcpyAsync(&bad, s->d_debug, sizeof(int), cudaMemcpyDeviceToHost, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  if (bad)
    return fail(s, SPH_ERR_STATE, "some targets' hits were not stored (overflow bits 0x%x)", bad);
  long long total = 0;
  for (int i = 0; i < n; ++i) {
    ho[i] = total;
    total += hc[i];
  }
  *count = total;
  if (cap == 0) return SPH_OK;
  CK(cudaMemcpyAsync(doff, ho.data(), 8 * (size_t)n, cudaMemcpyHostToDevice, s->stream));
  const long long m = total < cap ? total : cap;
  long long* dpairs = nullptr;
  if (cudaMalloc(&dpairs, 16 * (size_t)(m > 0 ? m : 1)) != cudaSuccess) {
    cudaGetLastError();
    return fail(s, SPH_ERR_NOMEM, "cannot allocate the pair list");
  }
  e = launch_debug_hits(ctx(s), s->cur, s->geo, s->b, s->n_host, mixed, 1, dcounts, doff, dpairs,
                        m, s->d_debug);
  cudaError_t e2 = cudaMemcpyAsync(pairs, dpairs, 16 * (size_t)m, cudaMemcpyDeviceToHost, s->stream);
  cudaError_t e3 = cudaStreamSynchronize(s->stream);
  cudaFree(dpairs);
  if (e != cudaSuccess || e2 != cudaSuccess || e3 != cudaSuccess)
    return fail(s, SPH_ERR_CUDA, "pair list transfer failed");
  return SPH_OK;
}

int sph_set_profiling(sph_system* s, int on) {
  if (!s) return SPH_ERR_ARG;
  s->profiling = on != 0;
  return SPH_OK;
}

int sph_kernel_stats(sph_system* s, int kernel, double* total_ms, int64_t* launches) {
  if (!s || kernel < 0 || kernel >= SPH_KERNEL_COUNT) return SPH_ERR_ARG;
  DeviceGuard guard(s->device);
  int rc = flush_profile(s);
  if (rc) return rc;
  if (total_ms) *total_ms = s->total_ms[kernel];
  if (launches) *launches = s->kernel_launches[kernel];
  return SPH_OK;
}

int sph_reset_kernel_stats(sph_system* s) {
  if (!s) return SPH_ERR_ARG;
  DeviceGuard guard(s->device);
  int rc = flush_profile(s);
  if (rc) return rc;
  for (int i = 0; i < SPH_KERNEL_COUNT; ++i) {
    s->total_ms[i] = 0.0;
    s->kernel_launches[i] = 0;
  }
  return SPH_OK;
}

int sph_set_tuning(sph_system* s, int warps_per_block) {
  if (!s) return SPH_ERR_ARG;
  if (warps_per_block != 2 && warps_per_block != 4 && warps_per_block != 8)
    return fail(s, SPH_ERR_ARG, "warps per block must be 2, 4 or 8 (got %d)", warps_per_block);
  if (s->k.warps != warps_per_block) ++s->generation;
  s->k.warps = warps_per_block;
  return SPH_OK;
}

int sph_get_tuning(const sph_system* s, int* warps_per_block) {
  if (!s || !warps_per_block) return SPH_ERR_ARG;
  *warps_per_block = s->k.warps;
  return SPH_OK;
}

int sph_set_chunk_threads(sph_system* s, int threads) {
  if (!s) return SPH_ERR_ARG;
  if (threads != 32 && threads != 64 && threads != 128)
    return fail(s, SPH_ERR_ARG, "threads per cell chunk must be 32, 64 or 128 (got %d)", threads);
  const int split = threads / 32;
  if (s->k.split != split) ++s->generation;
  s->k.split = split;
  return SPH_OK;
}

int sph_get_chunk_threads(const sph_system* s, int* threads) {
  if (!s || !threads) return SPH_ERR_ARG;
  *threads = 32 * s->k.split;
  return SPH_OK;
}

// Multiprocessors assumed by sph_memory_estimate (no CUDA call there): at
// least the count of any single GPU of this class, so the traversal scratch
// it adds is an upper bound.
constexpr int kEstimateSms = 160;

// The FP64 rows and pair list of n particles on the lattice the parameters
// imply (spacing dr = (m / rho0)^(1/dim)): every particle a full lattice
// neighbourhood within h (an interior fluid target -- walls and surface
// particles have fewer), rows padded to four entries, the headroom
// ensure_rows adds.  Only an estimate: a flow that clusters its particles
// needs more, and the rows then grow.
static size_t rows_estimate(const sph_params* p, long long n) {
  if (p->precision == SPH_PREC_MIXED || n <= 0) return 0;
  double dr = 0.0;
  if (p->mass > 0.0 && p->rho0 > 0.0) dr = std::pow(p->mass / p->rho0, 1.0 / p->dim);
  double ratio = dr > 0.0 ? p->h / dr : 4.0;
  if (!(ratio > 0.0) || ratio > 64.0) ratio = 4.0;
  const int R = (int)std::ceil(ratio);
  const double r2 = ratio * ratio * (1.0 + 1e-9);
  long long nb = 0;
  for (int i = -R; i <= R; ++i)
    for (int j = -R; j <= R; ++j)
      for (int k = (p->dim == 3 ? -R : 0); k <= (p->dim == 3 ? R : 0); ++k)
        if ((i || j || k) && (double)(i * i + j * j + k * k) <= r2) ++nb;
  const unsigned long long need = (unsigned long long)n * (unsigned long long)((nb + 3) & ~3LL);
  unsigned long long cap = std::min(need + need / 12 + 4096, kMaxRowEntries) & ~3ull;
  const unsigned long long pcap = cap / 2 + 1024;
  return align_up(sizeof(RowEntry) * cap) + 3 * align_up(4 * pcap);
}

int sph_memory_estimate(const sph_params* p, int64_t n, uint64_t* bytes) {
  if (!p || !bytes || n < 0 || n > 0x7fffffffLL - 64) return SPH_ERR_ARG;
  sph_system tmp;
  const int rc = setup_host(p, &tmp);
  if (rc) return rc;
  tmp.sms = kEstimateSms;
  *bytes = (uint64_t)(cells_bytes(&tmp) + carve(&tmp, nullptr, (size_t)(n > 0 ? n : 1)) +
                      rows_estimate(p, n));
  return SPH_OK;
}

int sph_memory_usage(const sph_system* s, uint64_t* bytes) {
  if (!s || !bytes) return SPH_ERR_ARG;
  sph_system tmp;
  tmp.params = s->params;
  tmp.geo = s->geo;
  tmp.sms = s->sms;
  size_t b = cells_bytes(s);
  if (s->arena) b += carve(&tmp, nullptr, (size_t)s->cap);
  b += s->rowbuf_bytes;
  b += s->query_bytes;
  *bytes = (uint64_t)b;
  return SPH_OK;
}

int sph_query(sph_system* s, int* idle) {
  if (!s || !idle) return SPH_ERR_ARG;
  DeviceGuard guard(s->device);
  const cudaError_t e = cudaStreamQuery(s->stream);
  if (e == cudaSuccess) {
    *idle = 1;
    return SPH_OK;
  }
  if (e == cudaErrorNotReady) {
    *idle = 0;
    return SPH_OK;
  }
  cudaGetLastError();
  return fail(s, SPH_ERR_CUDA, "stream query failed: %s", cudaGetErrorString(e));
}

int sph_launch_count(sph_system* s, int64_t* launches) {
  if (!s || !launches) return SPH_ERR_ARG;
  *launches = s->total_launches;
  return SPH_OK;
}


// ---------------------------------------------------------------- batches

static int bfail(sph_batch* b, int code, const char* msg) {
  if (b) b->err = msg;
  return code;
}

static void batch_drop_graph(sph_batch* b) {
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  b->exec = nullptr;
  b->graph = nullptr;
}

static void batch_hook(void* owner, int, int phase, int kernels) {
  if (phase == 1) ((sph_batch*)owner)->counted += kernels;
}

// Two steps of every member as one launch per kernel (sph_bin.cu, sph_pair32.cu,
// sph_unary.cu): argument arrays [0] (cur -> alt as the members hold them) and
// [1] (swapped); step 0 bins with [0] and runs the passes on [1], step 1 the
// other way round, so the ping-pong ends where it started, as two sph_steps do.
static int batch_capture_fused(sph_batch* b) {
  const int M = (int)b->members.size();
  std::vector<MemberArgs> args[2];
  for (int j = 0; j < M; ++j) {
    sph_system* m = b->members[j];
    MemberArgs a{};
    a.cur = m->cur;
    a.alt = m->alt;
    a.g = m->geo;
    a.k = m->k;
    a.b = m->b;
    a.cap = m->n_host;
    args[0].push_back(a);
    std::swap(a.cur, a.alt);
    args[1].push_back(a);
  }
  // the pair launches' warps per block: at least every member's split (a
  // block holds whole items of one member)
  int warps = b->fused_warps;
  for (int j = 0; j < M; ++j) warps = std::max(warps, b->members[j]->k.split);
  std::vector<int2> maps[kShapeCount];
  for (int sh = 0; sh < kShapeCount; ++sh)
    for (int j = 0; j < M; ++j) {
      const sph_system* m = b->members[j];
      const int nb = fused_blocks(sh, m->n_host, m->geo.key_max, m->b.max_items * m->k.split,
                                  warps);
      for (int i = 0; i < nb; ++i) maps[sh].push_back(make_int2(j, i));
    }
  size_t bytes = 2 * align_up(sizeof(MemberArgs) * M);
  for (int sh = 0; sh < kShapeCount; ++sh) bytes += align_up(sizeof(int2) * maps[sh].size());
  if (b->fdev) cudaFree(b->fdev);
  b->fdev = nullptr;
  if (cudaMalloc(&b->fdev, bytes) != cudaSuccess) {
    cudaGetLastError();
    return bfail(b, SPH_ERR_NOMEM, "cannot allocate the fused batch tables");
  }
  char* p = (char*)b->fdev;
  FusedBatch fb{};
  for (int q = 0; q < 2; ++q) {
    if (cudaMemcpy(p, args[q].data(), sizeof(MemberArgs) * M, cudaMemcpyHostToDevice) != cudaSuccess)
      return bfail(b, SPH_ERR_CUDA, "copying the member arguments failed");
    fb.args[q] = (const MemberArgs*)p;
    p += align_up(sizeof(MemberArgs) * M);
  }
  for (int sh = 0; sh < kShapeCount; ++sh) {
    if (cudaMemcpy(p, maps[sh].data(), sizeof(int2) * maps[sh].size(), cudaMemcpyHostToDevice) !=
        cudaSuccess)
      return bfail(b, SPH_ERR_CUDA, "copying the block tables failed");
    fb.map[sh] = (const int2*)p;
    fb.blocks[sh] = (int)maps[sh].size();
    p += align_up(sizeof(int2) * maps[sh].size());
  }
  fb.members = M;
  fb.dim = b->members[0]->params.dim;
  fb.warps = warps;
  fb.split = 0;
  for (int j = 0; j < M; ++j) fb.split |= b->members[j]->k.split > 1 ? 1 : 0;
  cudaError_t e = cudaStreamBeginCapture(b->origin, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return bfail(b, SPH_ERR_CUDA, "cudaStreamBeginCapture failed");
  b->counted = 0;
  const LaunchCtx c{b->origin, b, batch_hook};
  for (int step = 0; step < 2 && e == cudaSuccess; ++step) {
    const int q = 1 - step;  // the passes work on the gather's destination
    e = launch_fused_binning(c, fb, step);
    if (e == cudaSuccess) e = launch_fused_pair(c, fb, q, SPH_OP_DENSITY, 1, 1, 1, 1);
    if (e == cudaSuccess) e = launch_fused_pair(c, fb, q, SPH_OP_WALL_PRESSURE, 0, 0, 0, 0);
    if (e == cudaSuccess) e = launch_fused_pair(c, fb, q, SPH_OP_FORCE, 0, 1, 0, 2);
    if (e == cudaSuccess) e = launch_fused_unary(c, fb, q, SPH_OP_KICK);
  }
  cudaGraph_t g = nullptr;
  const cudaError_t e2 = cudaStreamEndCapture(b->origin, &g);
  if (e != cudaSuccess || e2 != cudaSuccess || !g) {
    cudaGetLastError();
    if (g) cudaGraphDestroy(g);
    return bfail(b, SPH_ERR_CUDA, "capturing the fused steps failed");
  }
  b->graph = g;
  if (cudaGraphInstantiate(&b->exec, g, 0) != cudaSuccess) {
    cudaGetLastError();
    batch_drop_graph(b);
    return bfail(b, SPH_ERR_CUDA, "cudaGraphInstantiate failed");
  }
  b->kernels_per_graph = b->counted;
  // the members' host-side view after two steps (sph_step's flags)
  for (int j = 0; j < M; ++j) {
    sph_system* m = b->members[j];
    m->cells_valid = true;
    m->aux_fluid = m->aux_wall = true;
    m->lists_valid = true;
    m->hits_valid = true;
    b->generations[j] = m->generation;
    b->cur0[j] = m->cur.x[0];
  }
  return SPH_OK;
}

// Captures two fused steps of every member into one graph.
static int batch_capture(sph_batch* b) {
  batch_drop_graph(b);
  if (b->fused) return batch_capture_fused(b);
  std::vector<long long> before(b->members.size());
  std::vector<bool> prof(b->members.size());
  for (size_t j = 0; j < b->members.size(); ++j) {
    before[j] = b->members[j]->total_launches;
    prof[j] = b->members[j]->profiling;
    b->members[j]->profiling = false;  // no event records inside the graph
  }
  cudaError_t e = cudaStreamBeginCapture(b->origin, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return bfail(b, SPH_ERR_CUDA, "cudaStreamBeginCapture failed");
  int rc = SPH_OK;
  cudaEventRecord(b->fork, b->origin);
  for (size_t j = 0; j < b->members.size() && !rc; ++j) {
    sph_system* m = b->members[j];
    cudaStreamWaitEvent(m->stream, b->fork, 0);
    rc = step_once(m);
    if (!rc) rc = step_once(m);
    cudaEventRecord(b->joins[j], m->stream);
    cudaStreamWaitEvent(b->origin, b->joins[j], 0);
  }
  cudaGraph_t g = nullptr;
  e = cudaStreamEndCapture(b->origin, &g);
  long long kernels = 0;
  for (size_t j = 0; j < b->members.size(); ++j) {
    kernels += b->members[j]->total_launches - before[j];
    b->members[j]->total_launches = before[j];  // captured, not yet executed
    b->members[j]->profiling = prof[j];
    b->generations[j] = b->members[j]->generation;
    b->cur0[j] = b->members[j]->cur.x[0];
  }
  if (rc) {
    if (g) cudaGraphDestroy(g);
    return bfail(b, rc, "a member's step failed during capture");
  }
  if (e != cudaSuccess || !g) return bfail(b, SPH_ERR_CUDA, "cudaStreamEndCapture failed");
  b->graph = g;
  if (cudaGraphInstantiate(&b->exec, g, 0) != cudaSuccess) {
    cudaGetLastError();
    batch_drop_graph(b);
    return bfail(b, SPH_ERR_CUDA, "cudaGraphInstantiate failed");
  }
  b->kernels_per_graph = kernels;
  return SPH_OK;
}

int sph_batch_create(sph_system* const* members, int count, sph_batch** out) {
  if (!members || !out || count <= 0) return SPH_ERR_ARG;
  *out = nullptr;
  for (int j = 0; j < count; ++j) {
    if (!members[j]) return SPH_ERR_ARG;
    if (members[j]->device != members[0]->device) return SPH_ERR_ARG;
    if (members[j]->n_host <= 0 || !members[j]->arena) return SPH_ERR_STATE;
    for (int i = 0; i < j; ++i)
      if (members[i] == members[j]) return SPH_ERR_ARG;
  }
  sph_batch* b = new sph_batch();
  b->members.assign(members, members + count);
  b->fusable = true;
  for (int j = 0; j < count; ++j)
    if (members[j]->params.precision != SPH_PREC_MIXED ||
        members[j]->params.dim != members[0]->params.dim)
      b->fusable = false;
  b->fused = b->fusable;
  b->generations.assign(count, -1);
  b->cur0.assign(count, nullptr);
  b->device = members[0]->device;
  DeviceGuard guard(b->device);
  bool ok = cudaStreamCreateWithFlags(&b->origin, cudaStreamNonBlocking) == cudaSuccess &&
            cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) == cudaSuccess &&
            cudaEventCreateWithFlags(&b->after, cudaEventDisableTiming) == cudaSuccess;
  b->joins.assign(count, nullptr);
  for (int j = 0; j < count && ok; ++j)
    ok = cudaEventCreateWithFlags(&b->joins[j], cudaEventDisableTiming) == cudaSuccess;
  if (!ok) {
    cudaGetLastError();
    sph_batch_destroy(b);
    return SPH_ERR_CUDA;
  }
  *out = b;
  return SPH_OK;
}

int sph_batch_destroy(sph_batch* b) {
  if (!b) return SPH_ERR_ARG;
  DeviceGuard guard(b->device);
  if (b->origin) cudaStreamSynchronize(b->origin);
  batch_drop_graph(b);
  if (b->fdev) cudaFree(b->fdev);
  for (auto e : b->joins)
    if (e) cudaEventDestroy(e);
  if (b->fork) cudaEventDestroy(b->fork);
  if (b->after) cudaEventDestroy(b->after);
  if (b->origin) cudaStreamDestroy(b->origin);
  delete b;
  return SPH_OK;
}

const char* sph_batch_last_error(const sph_batch* b) { return b ? b->err.c_str() : "null handle"; }

int sph_batch_step(sph_batch* b, int nsteps) {
  if (!b || nsteps < 0) return SPH_ERR_ARG;
  DeviceGuard guard(b->device);
  // FP64 members whose rows fell short in earlier steps grow them now (a
  // new generation: the graph is captured again)
  for (auto* m : b->members) {
    const int rc = grow_rows(m, false);
    if (rc) return bfail(b, rc, "growing a member's rows failed");
  }
  bool stale = !b->exec;
  for (size_t j = 0; j < b->members.size(); ++j)
    if (b->generations[j] != b->members[j]->generation ||
        b->cur0[j] != b->members[j]->cur.x[0])
      stale = true;
  if (nsteps >= 2 && stale) {
    // the members' own streams may still run earlier work: order after it
    for (auto* m : b->members) {
      cudaEventRecord(b->after, m->stream);
      cudaStreamWaitEvent(b->origin, b->after, 0);
    }
    const int rc = batch_capture(b);
    if (rc) return rc;
  }
  // the graph's branches start behind whatever each member queued before
  for (auto* m : b->members) {
    cudaEventRecord(b->after, m->stream);
    cudaStreamWaitEvent(b->origin, b->after, 0);
  }
  for (int it = 0; it + 1 < nsteps; it += 2) {
    if (cudaGraphLaunch(b->exec, b->origin) != cudaSuccess) {
      cudaGetLastError();
      return bfail(b, SPH_ERR_CUDA, "cudaGraphLaunch failed");
    }
    b->launches += b->kernels_per_graph;
    ++b->graph_launches;
  }
  // members continue on their own streams behind the graph
  cudaEventRecord(b->after, b->origin);
  for (auto* m : b->members) cudaStreamWaitEvent(m->stream, b->after, 0);
  if (nsteps & 1) {
    for (auto* m : b->members) {
      const long long l0 = m->total_launches;
      const int rc = step_once(m);
      if (rc) return bfail(b, rc, "a member's step failed");
      b->launches += m->total_launches - l0;
      m->total_launches = l0;
    }
  }
  return SPH_OK;
}

int sph_batch_set_fused(sph_batch* b, int on) {
  if (!b) return SPH_ERR_ARG;
  if (on && !b->fusable)
    return bfail(b, SPH_ERR_UNSUPPORTED, "fused steps need mixed-precision members of one dimension");
  if ((on != 0) != b->fused) {
    b->fused = on != 0;
    batch_drop_graph(b);  // captured again on the next step
  }
  return SPH_OK;
}

int sph_batch_set_tuning(sph_batch* b, int warps_per_block) {
  if (!b) return SPH_ERR_ARG;
  if (warps_per_block != 2 && warps_per_block != 4 && warps_per_block != 8)
    return bfail(b, SPH_ERR_ARG, "warps per block must be 2, 4 or 8");
  if (warps_per_block != b->fused_warps) {
    b->fused_warps = warps_per_block;
    if (b->fused) batch_drop_graph(b);
  }
  return SPH_OK;
}

int sph_batch_synchronize(sph_batch* b) {
  if (!b) return SPH_ERR_ARG;
  DeviceGuard guard(b->device);
  for (auto* m : b->members)
    if (cudaStreamSynchronize(m->stream) != cudaSuccess) return bfail(b, SPH_ERR_CUDA, "stream failed");
  if (cudaStreamSynchronize(b->origin) != cudaSuccess) return bfail(b, SPH_ERR_CUDA, "stream failed");
  return SPH_OK;
}

int sph_batch_stats(sph_batch* b, int64_t* kernels_per_graph, int64_t* graph_launches,
                    int64_t* kernels) {
  if (!b) return SPH_ERR_ARG;
  if (kernels_per_graph) *kernels_per_graph = b->kernels_per_graph;
  if (graph_launches) *graph_launches = b->graph_launches;
  if (kernels) *kernels = b->launches;
  return SPH_OK;
}

int sph_batch_query(sph_batch* b, int* idle) {
  if (!b || !idle) return SPH_ERR_ARG;
  DeviceGuard guard(b->device);
  int all = 1;
  std::vector<cudaStream_t> streams{b->origin};
  for (auto* m : b->members) streams.push_back(m->stream);
  for (cudaStream_t st : streams) {
    const cudaError_t e = cudaStreamQuery(st);
    if (e == cudaErrorNotReady) {
      all = 0;
    } else if (e != cudaSuccess) {
      cudaGetLastError();
      return bfail(b, SPH_ERR_CUDA, "stream query failed");
    }
  }
  *idle = all;
  return SPH_OK;
}

int sph_batch_stream(sph_batch* b, void** stream) {
  if (!b || !stream) return SPH_ERR_ARG;
  *stream = (void*)b->origin;
  return SPH_OK;
}

}  // extern "C"
