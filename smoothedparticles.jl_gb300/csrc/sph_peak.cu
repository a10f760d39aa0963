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

// int64 -> double conversions (round to nearest), 8 independent chains
__global__ void i2f_chains(double* out, int iters) {
  long long k[8];
  double d[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    k[j] = (long long)threadIdx.x * 7919 + j;
    d[j] = 0.0;
  }
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      d[j] = __ll2double_rn(k[j]);
      k[j] = __double_as_longlong(d[j]) ^ (long long)i;
    }
  }
  double s = 0.0;
#pragma unroll
  for (int j = 0; j < 8; ++j) s += d[j];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// 8 FP64 FMA chains with one int64 -> double conversion beside each FMA:
// at the FMA rate of fma_chains when the conversions take another pipe
__global__ void fma_i2f_chains(double* out, int iters, double a, double b) {
  double x[8], d[8];
  long long k[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    x[j] = threadIdx.x + j;
    k[j] = (long long)threadIdx.x * 7919 + j;
    d[j] = 0.0;
  }
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      x[j] = x[j] * a + b;
      d[j] = __ll2double_rn(k[j]);
      k[j] = __double_as_longlong(d[j]) ^ (long long)i;
    }
  }
  double s = 0.0;
#pragma unroll
  for (int j = 0; j < 8; ++j) s += x[j] + d[j];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace

extern "C" int sph_pipe_peak(int device, int which, double* instr_per_s) {
  if (!instr_per_s || which < 0 || which > 4) return SPH_ERR_ARG;
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
      else if (which == 2)
        add_chains<<<blocks, threads, 0, st>>>((double*)buf, iters, 1e-3);
      else if (which == 3)
        i2f_chains<<<blocks, threads, 0, st>>>((double*)buf, iters);
      else
        fma_i2f_chains<<<blocks, threads, 0, st>>>((double*)buf, iters, 0.999, 1e-3);
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
