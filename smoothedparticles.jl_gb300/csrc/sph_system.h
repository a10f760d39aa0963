// sph_system.h -- the handle behind the C ABI (private to the library):
// device memory, stream, cached flags, launch accounting.
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "sph_launch.h"
#include "sphgpu.h"

struct sph_system {
  using State = sphgpu::State;
  using Geometry = sphgpu::Geometry;
  using Consts = sphgpu::Consts;
  using BinScratch = sphgpu::BinScratch;
  sph_params params{};
  int device = 0;
  Geometry geo{};
  Consts k{};
  cudaStream_t stream = nullptr;
  State cur{}, alt{};
  BinScratch b{};
  void* arena = nullptr;    // per-particle arrays (both SoA sets + scratch + staging)
  void* cells = nullptr;    // cell tables and counters
  void* staging = nullptr;  // host-transfer staging inside the arena
  double* query = nullptr;  // sum() query buffer
  size_t query_bytes = 0;
  int cap = 0;              // particles the arena holds
  int sms = 1;              // multiprocessors of the device
  // FP64 systems: the rows and the pair list (their own allocation, grown
  // to a high-water mark of what the passes needed) and the host-mapped word
  // the passes report a shortfall in
  void* rowbuf = nullptr;
  size_t rowbuf_bytes = 0;
  unsigned long long* need_host = nullptr;
  bool rows_impossible = false;  // more entries than 32-bit offsets address
  int n_host = 0;           // upper bound of the device-resident count
  bool cells_valid = false;
  // FP32 neighbour records current (mixed precision): of the fluid particles
  // (written by a fused density pass) and of the walls (wall-pressure pass)
  bool aux_fluid = false;
  bool aux_wall = false;
  bool lists_valid = false;  // hit lists of the last density pass match cells and positions
  // the neighbour indices the last density pass stored (FP64 rows, mixed hit
  // masks) belong to the current cells: sph_debug_hits may read them
  bool hits_valid = false;
  int* d_debug = nullptr;    // a device word of the debug listings (in the cell tables)
  std::string err;
  // launch accounting and optional per-kernel CUDA-event timing
  bool profiling = false;
  struct Pending {
    int kid;
    cudaEvent_t start, stop;
  };
  std::vector<Pending> pending;
  std::vector<cudaEvent_t> pool;
  cudaEvent_t open_start = nullptr;
  double total_ms[SPH_KERNEL_COUNT] = {};
  long long kernel_launches[SPH_KERNEL_COUNT] = {};
  long long total_launches = 0;
  // bumped whenever device buffers are reallocated or the launch shape
  // changes, so a batch knows its captured graph is stale
  long long generation = 0;
  // sph_step's captured two-step graph (a batch of this system alone)
  sph_batch* solo = nullptr;
  // sph_step_io: the stream its reads run on and the events they wait for
  // (after the binning, after the wall pressure, at the end of the step)
  cudaStream_t io_stream = nullptr;
  cudaEvent_t io_ev[3] = {nullptr, nullptr, nullptr};
};

namespace sphgpu {

// Makes `dev` current for the guard's lifetime.
struct DeviceGuard {
  int prev = -1;
  explicit DeviceGuard(int dev) {
    cudaGetDevice(&prev);
    if (prev != dev) cudaSetDevice(dev);
  }
  ~DeviceGuard() {
    int cur = -1;
    cudaGetDevice(&cur);
    if (prev >= 0 && cur != prev) cudaSetDevice(prev);
  }
};

// The system's launch context (stream + launch accounting / profiling hook).
LaunchCtx system_ctx(sph_system* s);
// Records msg as the system's last error; returns code.
int system_fail(sph_system* s, int code, const char* msg);

}  // namespace sphgpu
