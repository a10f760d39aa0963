// sph_peak.cu -- issue-rate microbenchmark of the FP64 and FP32 pipes, the
// denominators of the pair passes' roofline (GB300 has no FP64 tensor path
// worth using and the pair passes are not contractions).
#include <cuda_runtime.h>

#include "sphgpu.h"

namespace {

template <typename T>
__global__ void fma_chains(T* out, int iters, T a, T b) {
  T x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3;
  T x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
    x0 = x0 * a + b; x1 = x1 * a + b; x2 = x2 * a + b; x3 = x3 * a + b;
    x4 = x4 * a + b; x5 = x5 * a + b; x6 = x6 * a + b; x7 = x7 * a + b;
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

__global__ void add_chains(double* out, int iters, double b) {
  double x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3;
  double x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
    x0 = x0 + b; x1 = x1 + b; x2 = x2 + b; x3 = x3 + b;
    x4 = x4 + b; x5 = x5 + b; x6 = x6 + b; x7 = x7 + b;
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

}  // namespace

extern "C" int sph_pipe_peak(int device, int which, double* instr_per_s) {
  if (!instr_per_s || which < 0 || which > 2) return SPH_ERR_ARG;
  int prev = 0;
  if (cudaGetDevice(&prev) != cudaSuccess || cudaSetDevice(device) != cudaSuccess) {
    cudaGetLastError();
    return SPH_ERR_CUDA;
  }
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  const int threads = 256, blocks = sms * 8;
  const size_t n = (size_t)blocks * threads;
  void* buf = nullptr;
  cudaStream_t st = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int rc = SPH_OK;
  if (cudaMalloc(&buf, n * sizeof(double)) != cudaSuccess || cudaStreamCreate(&st) != cudaSuccess ||
      cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
    rc = SPH_ERR_CUDA;
  } else {
    const int iters = which == 1 ? 100000 : 2000;
    float best = 1e30f;
    for (int rep = 0; rep < 3; ++rep) {
      cudaEventRecord(e0, st);
      if (which == 0)
        fma_chains<double><<<blocks, threads, 0, st>>>((double*)buf, iters, 0.999, 1e-3);
      else if (which == 1)
        fma_chains<float><<<blocks, threads, 0, st>>>((float*)buf, iters, 0.999f, 1e-3f);
      else
        add_chains<<<blocks, threads, 0, st>>>((double*)buf, iters, 1e-3);
      cudaEventRecord(e1, st);
      float ms = 0.f;
      if (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) {
        rc = SPH_ERR_CUDA;
        break;
      }
      if (ms < best) best = ms;
    }
    if (rc == SPH_OK) *instr_per_s = (double)n * 8.0 * iters / (best * 1e-3);
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (st) cudaStreamDestroy(st);
  if (buf) cudaFree(buf);
  cudaGetLastError();
  cudaSetDevice(prev);
  return rc;
}
