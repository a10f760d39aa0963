// sph_launch.h -- host-side launchers of the device kernels (one per kernel
// family); the C ABI in sph_api.cu strings them together.
#pragma once

#include <vector>

#include "sph_common.cuh"
#include "sphgpu.h"

namespace sphgpu {

// Launch context: the stream plus an optional hook called around every kernel
// launch (profiling events and the launch counter live in the API layer).
struct LaunchCtx {
  cudaStream_t stream;
  void* owner;
  // phase 0 before the launches of one kernel family, phase 1 after them;
  // `kernels` (phase 1 only) is how many kernels were launched in between.
  void (*mark)(void* owner, int kernel, int phase, int kernels);
};

inline void mark(const LaunchCtx& c, int kernel, int phase, int kernels = 1) {
  if (c.mark) c.mark(c.owner, kernel, phase, kernels);
}

// Blocks of one resident wave of `kernel` on the current device (kernels
// whose warps stride over their work launch this many: blocks beyond the
// resident ones would only start after the first wave).
template <class K>
int resident_blocks(K kernel, int threads) {
  int dev = 0, sms = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, 0);
  cudaGetLastError();
  return (sms > 0 ? sms : 1) * (per_sm > 0 ? per_sm : 1);
}

// Fields moved by the reorder gather.
constexpr int kGatherAll = 1;   // every field (create_cell_list!)
constexpr int kGatherStep = 0;  // only what survives a fused step (x, v, rho_ref, ids)

// ---- fused batches: one launch per kernel of the step for all members.
// Members' launch arguments live in device memory; for every launch shape a
// table gives each block its (member, block of that member).
struct MemberArgs {
  State cur;      // the state the step starts from
  State alt;      // the binning's gather destination (the pair passes' state)
  Geometry g;
  Consts k;
  BinScratch b;
  int cap;        // particle capacity (the count upper bound)
};

enum FusedShape {
  kShapeParticles = 0,  // ceil(cap / 256) blocks of 256 threads
  kShapeBuckets,        // ceil((key_max + 3) / 256)
  kShapeCells,          // ceil(key_max / 256)
  kShapeRank,           // ceil(key_max / 8): one warp per cell
  kShapeScanTiles,      // ceil((key_max + 3) / 4096): scan tiles
  kShapeMember,         // one block per member
  kShapeItems,          // ceil(max_items / warps): the pair passes' warps
  kShapeCount
};

struct FusedBatch {
  const MemberArgs* args[2];  // [0]: cur -> alt as given; [1]: cur and alt swapped
  const int2* map[kShapeCount];
  int blocks[kShapeCount];
  int members;
  int dim;
  int warps;  // warps per block of the fused pair passes (2, 4 or 8)
  int split;  // some member shares its work items between warps (chunk threads > 32)
};

// Blocks of each shape for one member (the single-system launch grids).
int fused_blocks(int shape, int cap, int key_max, int max_items, int warps);
// The binning of one fused step for every member (sph_bin.cu): args[p].cur ->
// args[p].alt; the pair passes (sph_pair32.cu) and the kick (sph_unary.cu) of
// the step then work on args[1 - p].cur (= args[p].alt).
cudaError_t launch_fused_binning(const LaunchCtx& c, const FusedBatch& fb, int p);
cudaError_t launch_fused_pair(const LaunchCtx& c, const FusedBatch& fb, int p, int op, int self,
                              int reset, int fuse_eos, int list_mode);
cudaError_t launch_fused_unary(const LaunchCtx& c, const FusedBatch& fb, int p, int op);

// ---- binning (sph_bin.cu)
// Whole create_cell_list!: keys (optionally with the fused kick + drift),
// removal replay, counting sort by cell, per-cell descending reference-index
// order, reorder gather cur -> alt.  `cap` bounds the particle count.
cudaError_t launch_binning(const LaunchCtx& c, const State& cur, const State& alt,
                           const Geometry& g, const Consts& k, const BinScratch& b, int cap,
                           int step_mode, int gather_mode);
// Exclusive prefix sum of len ints (in and out may not alias).
cudaError_t launch_scan(const LaunchCtx& c, const int* in, int* out, int len, int* tmp);
size_t scan_tmp_ints(int len);

// ---- FP64 pair passes (sph_pair64.cu)
// op: SPH_OP_DENSITY / SPH_OP_DENSITY_REF / SPH_OP_FORCE.  reset: start the
// accumulators at 0 (the folded reset_*! of a step) instead of the stored
// values; fuse_eos: apply the Tait EOS in the density epilogue.
// lists_valid: the rows of the last density pass belong to the current
// binning and positions, so the force pass may evaluate into them instead of
// traversing.
cudaError_t launch_pair_fp64(const LaunchCtx& c, const State& s, const Geometry& g,
                             const Consts& k, const BinScratch& b, int cap, int op, int self,
                             int reset, int fuse_eos, int lists_valid);
// ---- FP64 pair evaluation once per pair (sph_tile64.cu)
// phase 0 (density pass): counts, row lengths, the rows' scan and segment
// offsets, m W and distances into the rows; phase 1 (force pass, after the
// density pass of the same binning): the force records, then pressure and
// XSPH factors into the rows.  Launches kTilesLaunches[phase] kernels.
constexpr int kTilesLaunches[2] = {7, 2};
// launches of the density (0) and force (1) passes of a step: the tile
// kernels, the row sums and the traversal of overflowed rows
constexpr int kRowPassLaunches[2] = {kTilesLaunches[0] + 2, kTilesLaunches[1] + 2};
cudaError_t launch_tiles_fp64(const LaunchCtx& c, const State& s, const Geometry& g,
                              const Consts& k, const BinScratch& b, int cap, int phase);
// ---- mixed-precision pair passes (sph_pair32.cu)
// aux_fresh: the FP32 neighbour copies (vr, rhof) of the fluid particles are
// current (written by a fused density pass since the last state change);
// otherwise the wall-pressure and force passes rebuild them first.
cudaError_t launch_pair_mixed(const LaunchCtx& c, const State& s, const Geometry& g,
                              const Consts& k, const BinScratch& b, int cap, int op, int self,
                              int reset, int fuse_eos, int aux_fresh, int lists_valid);
// sum(sys, func, x) at nq device points (x: nq x 3) or, when rid_query is not
// null, at particles given by reference index.
cudaError_t launch_sum(const LaunchCtx& c, const State& s, const Geometry& g, const Consts& k,
                       const BinScratch& b, int func, int nq, const double* x,
                       const long long* rid_query, double* out);
// Neighbour pairs in the reference order: pass 0 counts per reference index,
// pass 1 writes (rid_p, rid_q) at offsets[rid_p].
cudaError_t launch_debug_pairs(const LaunchCtx& c, const State& s, const Geometry& g,
                               const Consts& k, const BinScratch& b, int cap, int pass,
                               int* counts, const long long* offsets, long long* pairs,
                               long long cap_pairs);

// The pairs the last density pass stored (FP64 rows or mixed hit masks) in
// the reference order: pass 0 counts per reference index, pass 1 writes;
// *bad (device) gets a bit when some target's hits were not stored.
cudaError_t launch_debug_hits(const LaunchCtx& c, const State& s, const Geometry& g,
                              const BinScratch& b, int cap, int mixed, int pass, int* counts,
                              const long long* offsets, long long* pairs, long long cap_pairs,
                              int* bad);

// ---- device-side particle generation (sph_lattice.cu)
struct LatticeShape {
  int kind, type, dim, keep_axis;
  double dr, lo[3], hi[3], keep_max;
  long long i0[3], n[3];  // first lattice index and count per axis (n[2] = 1 in 2D)
  int n_off;              // ball offsets of a boundary layer
};
// Validates a shape and fills the kernels' description plus the layer's ball
// offsets (x, y, z triples), computed on the host.
int lattice_prepare(const sph_shape& in, int dim, LatticeShape& out, std::vector<double>& offs);
long long lattice_points(const LatticeShape& s);
// flags[idx] = 1 for the lattice points of the shape (idx in loop order)
cudaError_t launch_lattice_flags(const LaunchCtx& c, const LatticeShape& s, const double* offs,
                                 int* flags);
// point idx with flags[idx] goes to row base + pos[idx] of x (n x 3) and type
cudaError_t launch_lattice_write(const LaunchCtx& c, const LatticeShape& s, const int* flags,
                                 const int* pos, double* x, int* type, int base);

// ---- unary operators and field transfer (sph_unary.cu)
cudaError_t launch_unary(const LaunchCtx& c, const State& s, const Consts& k,
                         const BinScratch& b, int cap, int op);
// Upload: staging (reference order, AoS n x 3 for vectors) -> SoA state.
cudaError_t launch_upload(const LaunchCtx& c, const State& s, const Consts& k,
                          const BinScratch& b, int n, const double* x, const double* v,
                          const double* rho, const double* rho_ref, const int* type);
// Field copy between the SoA state and a reference-ordered staging buffer.
// dir 0: state -> staging, 1: staging -> state.
cudaError_t launch_field(const LaunchCtx& c, const State& s, const Consts& k,
                         const BinScratch& b, int cap, int field, int dir, void* staging);

}  // namespace sphgpu
