// sph_noalloc.cu -- sph_cell_list_noalloc: the cell-list build (binning) for
// callers that cannot let a library allocate device memory.
//
// Who needs it: a host whose device memory is owned by its own pool or budget
// (e.g. a Julia program whose CUDA.jl allocator tracks and reuses every byte,
// or a serving process that admits work against a fixed HBM budget) cannot
// have a library call cudaMalloc behind its back -- the hidden allocation
// escapes the pool's accounting, can fail in the middle of a run, and
// cudaMalloc/cudaFree synchronise the device.  This entry point therefore
// allocates nothing: the caller passes inputs and outputs, and the scratch of
// the counting sort lives in one file-scope static device array of fixed size
// that every GPU which loads the library holds until the process exits.
//
// Output, identical to what create_cell_list! (core.jl:51-90) builds when no
// particle is removed: cell k (1-based key, structs.jl:97-106) holds
// order[cell_start[k] .. cell_start[k+1]), particle indices in descending
// order (core.jl:26-41).  Particles outside the domain's bounding box (NaN
// included) are not binned: they follow in order[cell_start[key_max+1] .. n),
// also in descending index order, for the caller to remove.
#include <cuda.h>

#include <cmath>
#include <mutex>

#include "sph_launch.h"
#include "sphgpu.h"

namespace sphgpu {
namespace {

constexpr int kMaxN = SPH_NOALLOC_MAX_PARTICLES;
constexpr int kMaxCells = SPH_NOALLOC_MAX_CELLS;
constexpr int kBuckets = kMaxCells + 3;  // cells 1..key_max, removed, total
constexpr int kScanTmp = 1024;           // >= scan_tmp_ints(kBuckets)
// keys | slots | bucketed indices | counts | starts | scan block sums
constexpr size_t kScratchInts = 3 * (size_t)kMaxN + 2 * (size_t)kBuckets + kScanTmp;

// The shared scratch.  Host code must not take its address directly (the
// symbol is a host-side stand-in); the device address comes from
// cudaGetSymbolAddress below.
static __device__ __align__(256) int g_noalloc_scratch[kScratchInts];

constexpr int kThreads = 256;

struct Geo {
  double h;
  double dmin[3], dmax[3];
  long long key_phase[3], key_lim[3];
  int key_max;
};

__global__ void __launch_bounds__(kThreads) na_keys(const double* __restrict__ x, int n, Geo g,
                                                    int* keys, int* slots, int* counts) {
  const int i = blockIdx.x * kThreads + threadIdx.x;
  if (i >= n) return;
  double p[3] = {x[3 * i], x[3 * i + 1], x[3 * i + 2]};
  bool inside = true;
#pragma unroll
  for (int d = 0; d < 3; ++d) inside = inside && (g.dmin[d] <= p[d]) && (p[d] <= g.dmax[d]);
  int key = g.key_max + 1;
  if (inside) {
    long long ijk[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) ijk[d] = 1 + (long long)floor(p[d] / g.h) - g.key_phase[d];
    const long long kk =
        ijk[0] + g.key_lim[0] * (ijk[1] - 1) + g.key_lim[0] * g.key_lim[1] * (ijk[2] - 1);
    if (kk >= 1 && kk <= g.key_max) key = (int)kk;
  }
  keys[i] = key;
  const unsigned active = __activemask();
  const unsigned peers = __match_any_sync(active, key);
  const int leader = __ffs(peers) - 1;
  int base = 0;
  if ((int)(threadIdx.x & 31) == leader) base = atomicAdd(&counts[key], __popc(peers));
  base = __shfl_sync(peers, base, leader);
  slots[i] = base + __popc(peers & lanemask_lt());
}

__global__ void __launch_bounds__(kThreads) na_scatter(int n, const int* keys, const int* slots,
                                                       const int* starts, int* bucketed) {
  const int i = blockIdx.x * kThreads + threadIdx.x;
  if (i >= n) return;
  bucketed[starts[keys[i]] + slots[i]] = i;
}

// flags of the particles outside the domain (reuses the slots array)
__global__ void __launch_bounds__(kThreads) na_flags(int n, int sentinel, const int* keys,
                                                     int* flags) {
  const int i = blockIdx.x * kThreads + threadIdx.x;
  if (i < n) flags[i] = keys[i] == sentinel;
}

// excluded particles after the binned ones, descending: the one with the
// largest index first.  below[i] = excluded particles with a smaller index.
__global__ void __launch_bounds__(kThreads) na_place_excluded(int n, int sentinel, const int* keys,
                                                              const int* below, const int* starts,
                                                              int* order) {
  const int i = blockIdx.x * kThreads + threadIdx.x;
  if (i >= n || keys[i] != sentinel) return;
  const int n_in = starts[sentinel];
  const int excluded = n - n_in;
  order[n_in + (excluded - 1 - below[i])] = i;
}

// one warp per cell: slot of an index = number of indices of the cell larger
// than it (cells hold tens of particles)
__global__ void __launch_bounds__(kThreads) na_rank(int nbuckets, const int* starts,
                                                    const int* bucketed, int* order) {
  const int lane = threadIdx.x & 31;
  const int bucket = blockIdx.x * (kThreads / 32) + (threadIdx.x >> 5) + 1;
  if (bucket > nbuckets) return;
  const int st = starts[bucket];
  const int en = starts[bucket + 1];
  for (int e = st + lane; e < en; e += 32) {
    const int my = bucketed[e];
    int rank = 0;
    for (int f = st; f < en; ++f) rank += (bucketed[f] > my);
    order[st + rank] = my;
  }
}

__global__ void na_copy_starts(int len, const int* starts, int* out) {
  const int i = blockIdx.x * kThreads + threadIdx.x;
  if (i < len) out[i] = starts[i];
}

// Device address of the scratch, looked up once per CUDA context.  A context
// that is destroyed and created again (cudaDeviceReset, CUDA.jl's
// device_reset!) loads the module again, possibly at another address, so the
// cache is keyed by the context's process-unique id (cuCtxGetId), not by the
// device number.  The two driver functions are fetched through the runtime's
// entry-point query, so the library does not link libcuda directly.
using CtxGetCurrent = CUresult (*)(CUcontext*);
using CtxGetId = CUresult (*)(CUcontext, unsigned long long*);

struct ScratchSlot {
  unsigned long long ctx_id;
  int* addr;
};

std::mutex g_mu;
CtxGetCurrent g_get_current = nullptr;
CtxGetId g_get_id = nullptr;
bool g_driver_ready = false;
constexpr int kSlots = 64;
ScratchSlot g_slots[kSlots] = {};
int g_next_slot = 0;

int driver_functions() {
  if (g_driver_ready) return SPH_OK;
  void* f1 = nullptr;
  void* f2 = nullptr;
  cudaDriverEntryPointQueryResult q1 = cudaDriverEntryPointSymbolNotFound, q2 = q1;
  if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1) !=
          cudaSuccess ||
      cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) !=
          cudaSuccess ||
      q1 != cudaDriverEntryPointSuccess || q2 != cudaDriverEntryPointSuccess || !f1 || !f2) {
    cudaGetLastError();
    return SPH_ERR_CUDA;
  }
  g_get_current = (CtxGetCurrent)f1;
  g_get_id = (CtxGetId)f2;
  g_driver_ready = true;
  return SPH_OK;
}

int scratch_on_current_device(int** out) {
  std::lock_guard<std::mutex> lock(g_mu);
  if (driver_functions() != SPH_OK) return SPH_ERR_CUDA;
  CUcontext ctx = nullptr;
  if (g_get_current(&ctx) != CUDA_SUCCESS) return SPH_ERR_CUDA;
  if (!ctx) {
    // no context current on this thread yet: the runtime's own choice, the
    // current device's primary context (cudaSetDevice initialises it)
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaSetDevice(dev) != cudaSuccess) {
      cudaGetLastError();
      return SPH_ERR_CUDA;
    }
    if (g_get_current(&ctx) != CUDA_SUCCESS || !ctx) return SPH_ERR_CUDA;
  }
  unsigned long long id = 0;
  if (g_get_id(ctx, &id) != CUDA_SUCCESS) return SPH_ERR_CUDA;
  for (const ScratchSlot& sl : g_slots)
    if (sl.addr && sl.ctx_id == id) {
      *out = sl.addr;
      return SPH_OK;
    }
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess || !p) {
    cudaGetLastError();
    return SPH_ERR_CUDA;
  }
  // contexts beyond kSlots reuse the oldest slot (a lookup again costs little)
  g_slots[g_next_slot] = ScratchSlot{id, (int*)p};
  g_next_slot = (g_next_slot + 1) % kSlots;
  *out = (int*)p;
  return SPH_OK;
}

}  // namespace
}  // namespace sphgpu

using namespace sphgpu;

extern "C" int sph_cell_list_noalloc(const sph_params* params, int64_t n, const double* d_x,
                                     int32_t* d_cell_start, int32_t* d_order, void* stream) {
  if (!params || n < 0 || (n > 0 && (!d_x || !d_order)) || !d_cell_start) return SPH_ERR_ARG;
  // the same checks as sph_create (structs.jl:59 asserts h > 0)
  if (params->dim != 2 && params->dim != 3) return SPH_ERR_ARG;
  if (!(params->h > 0.0)) return SPH_ERR_ARG;
  if (n > kMaxN) return SPH_ERR_BUDGET;  // more particles than the static scratch holds
  if (params->dim == 2 && (params->domain_min[2] > 0.0 || params->domain_max[2] < 0.0))
    return SPH_ERR_ARG;  // a 2D domain contains the plane z = 0
  Geo g{};
  g.h = params->h;
  long long key_max = 1;
  for (int d = 0; d < 3; ++d) {
    if (!(params->domain_min[d] <= params->domain_max[d])) return SPH_ERR_ARG;
    g.dmin[d] = params->domain_min[d];
    g.dmax[d] = params->domain_max[d];
    // floor(domain / h) must be a representable cell index before any
    // product is formed: a tiny h against the domain is a table too large
    const double lo = std::floor(params->domain_min[d] / g.h);
    const double hi = std::floor(params->domain_max[d] / g.h);
    if (!(lo >= -4.0e15 && hi <= 4.0e15)) return SPH_ERR_BUDGET;
    g.key_phase[d] = (long long)lo;
    g.key_lim[d] = (long long)hi - g.key_phase[d] + 1;
    if (g.key_lim[d] < 1 || g.key_lim[d] > kMaxCells) return SPH_ERR_BUDGET;
    key_max *= g.key_lim[d];
    if (key_max > kMaxCells) return SPH_ERR_BUDGET;  // cell table too large
  }
  g.key_max = (int)key_max;
  int* base = nullptr;
  int rc = scratch_on_current_device(&base);
  if (rc) return rc;
  int* keys = base;
  int* slots = keys + kMaxN;
  int* bucketed = slots + kMaxN;
  int* counts = bucketed + kMaxN;
  int* starts = counts + kBuckets;
  int* scan_tmp = starts + kBuckets;
  cudaStream_t st = (cudaStream_t)stream;
  const int nb = g.key_max + 3;
  const int N = (int)n;
  const int blocks = N > 0 ? (N + kThreads - 1) / kThreads : 1;
  // the scratch keeps the previous call's contents: the counts must start at 0
  if (cudaMemsetAsync(counts, 0, sizeof(int) * (size_t)nb, st) != cudaSuccess) {
    cudaGetLastError();
    return SPH_ERR_CUDA;
  }
  if (N > 0) na_keys<<<blocks, kThreads, 0, st>>>(d_x, N, g, keys, slots, counts);
  const LaunchCtx c{st, nullptr, nullptr};
  cudaError_t e = launch_scan(c, counts, starts, nb, scan_tmp);
  if (e == cudaSuccess && N > 0) {
    na_scatter<<<blocks, kThreads, 0, st>>>(N, keys, slots, starts, bucketed);
    const int ncells = g.key_max;
    na_rank<<<(ncells + kThreads / 32 - 1) / (kThreads / 32), kThreads, 0, st>>>(
        ncells, starts, bucketed, d_order);
    // particles outside the domain, in descending index order after the rest
    const int sentinel = g.key_max + 1;
    na_flags<<<blocks, kThreads, 0, st>>>(N, sentinel, keys, slots);
    e = launch_scan(c, slots, bucketed, N, scan_tmp);
    if (e == cudaSuccess)
      na_place_excluded<<<blocks, kThreads, 0, st>>>(N, sentinel, keys, bucketed, starts, d_order);
  }
  if (e == cudaSuccess) {
    const int len = g.key_max + 2;
    na_copy_starts<<<(len + kThreads - 1) / kThreads, kThreads, 0, st>>>(len, starts, d_cell_start);
    e = cudaGetLastError();
  }
  if (e != cudaSuccess) {
    cudaGetLastError();
    return SPH_ERR_CUDA;
  }
  return SPH_OK;
}
