// sph_assemble.cu -- assemble_matrix / assemble_vector (src/core.jl:164-225)
// on the device, as a CSR matrix in reference particle order, and the
// conjugate-gradient solve the implicit example applies to it
// (examples/collapse_dry_implicit.jl:218-233, IterativeSolvers.cg).
//
// Matrix: every row p (reference index) holds one entry per particle q within
// the support, q = p included (core.jl:210-213 keeps it, with r = 0).
//   1. count: one thread per particle walks the 3^d cells in key_diff order
//      and counts; the row offsets are an exclusive scan of the counts;
//      every walk classifies its candidates with the pair passes' FP32
//      pre-test first and forms the FP64 distance only for hits and band
//      candidates (the decision equals the reference's r > h test);
//   2. fill: the same walk writes (reference index of q, value) in the
//      reference's push order; the projection matrix's diagonal needs the
//      row's div_L_lambda! sums, formed first in the same order;
//   3. sort: one warp per row ranks the row's entries by column (columns are
//      unique within a row) -- the canonical CSR of sparse(I, J, V).
// Values are FP64 with the reference's expression order (this unit is built
// with --fmad=false), so they equal the CPU restatement bit for bit.
//
// CG (unpreconditioned, x0 = 0, stop when ||r|| <= reltol ||b||): SpMV with
// one warp per row; dot products reduced in a fixed order (per-block partials
// over a fixed grid, then one block), so a solve is reproducible.
#include <cmath>
#include <cstdint>
#include <vector>

#include "sph_launch.h"
#include "sph_system.h"
#include "sphgpu.h"

using namespace sphgpu;

namespace {

constexpr int kThreads = 128;
constexpr int kDotBlocks = 304;  // 2 per SM

// r = sqrt((d0 d0 + d1 d1) + d2 d2), d = x_p - x_q (core.jl:8-10)
template <int DIM>
__device__ __forceinline__ double dist64(const State& s, const double* xp, int q, double* d) {
  d[0] = xp[0] - s.x[0][q];
  d[1] = xp[1] - s.x[1][q];
  d[2] = DIM == 3 ? xp[2] - s.x[2][q] : 0.0;
  double ss = d[0] * d[0] + d[1] * d[1];
  if (DIM == 3) ss = ss + d[2] * d[2];
  return sqrt(ss);
}

// The pair passes' FP32 pre-test on cell-relative positions (the target at
// (ax, ay, az) relative to the candidate's cell): 1 inside the support,
// 0 beyond it, -1 in the band around r = h where the reference's FP64 test
// decides.  Outside the band the FP32 decision equals the FP64 one, so the
// FP64 distance is formed only for the hits and the band.
template <int DIM>
__device__ __forceinline__ int pre_test(const Consts& k, float ax, float ay, float az,
                                        const float4& q) {
  const float dx = ax - q.x, dy = ay - q.y;
  float ss = dx * dx + dy * dy;
  if (DIM == 3) {
    const float dz = az - q.z;
    ss = ss + dz * dz;
  }
  return ss > k.s_hi ? 0 : ss < k.s_lo ? 1 : -1;
}

// Particle i's position relative to neighbour cell nk (its own cell-relative
// position minus the cell's offset, as the pair passes form it).
__device__ __forceinline__ float4 rel_to(const Geometry& g, const Consts& k, const float4& pi,
                                         int cx, int cy, int cz, int nk) {
  int qx, qy, qz;
  decode_key(g, nk, qx, qy, qz);
  return make_float4(pi.x - (float)(qx - cx) * k.cellf, pi.y - (float)(qy - cy) * k.cellf,
                     pi.z - (float)(qz - cz) * k.cellf, 0.f);
}

// div_L_lambda! (collapse_dry_implicit.jl:140-145) of particle i over its
// neighbours q != i in the reference order, after initialize! (div = L = 0,
// lambda = 1)
template <int DIM>
__device__ void div_L_lambda(const State& s, const Geometry& g, const Consts& k, const BinScratch& b,
                             int i, double& div, double& L, double& lam) {
  const int key = s.cell[i];
  double xp[3] = {s.x[0][i], s.x[1][i], DIM == 3 ? s.x[2][i] : 0.0};
  double vp[3] = {s.v[0][i], s.v[1][i], DIM == 3 ? s.v[2][i] : 0.0};
  const double m = k.mass, rho = k.rho0, dim = (double)DIM;
  double dv = 0.0, l = 0.0, la = 1.0;
  const float4 pi = s.pl[i];
  int cx, cy, cz;
  decode_key(g, key, cx, cy, cz);
  for (int c = 0; c < g.n_diff; ++c) {
    const int nk = key + g.key_diff[c];
    if (nk < 1 || nk > g.key_max) continue;
    const float4 a = rel_to(g, k, pi, cx, cy, cz, nk);
    for (int q = b.cell_start[nk]; q < b.cell_start[nk + 1]; ++q) {
      const int pt = pre_test<DIM>(k, a.x, a.y, a.z, __ldg(&s.pl[q]));
      if (pt == 0 || q == i) continue;
      double d[3];
      const double r = dist64<DIM>(s, xp, q, d);
      if (pt < 0 && r > k.h) continue;
      const double rDk = ker_rdw(k, r);
      const double w0 = vp[0] - s.v[0][q];
      const double w1 = vp[1] - s.v[1][q];
      double dot = d[0] * w0 + d[1] * w1;
      if (DIM == 3) dot = dot + d[2] * (vp[2] - s.v[2][q]);
      dv = dv + ((-dot) * m) * rDk;
      l = l + ((-2.0 * m) / rho) * rDk;
      la = la + (((m / rho) * rDk) * (r * r)) / dim;
    }
  }
  div = dv;
  L = l;
  lam = la;
}

template <int DIM>
__global__ void __launch_bounds__(kThreads) asm_count_kernel(State s, Geometry g, Consts k,
                                                             BinScratch b, int* row_nnz) {
  const int n = *b.d_n;
  const int i = blockIdx.x * kThreads + threadIdx.x;
  if (i >= n) return;
  const int key = s.cell[i];
  double xp[3] = {s.x[0][i], s.x[1][i], DIM == 3 ? s.x[2][i] : 0.0};
  int cnt = 0;
  const float4 pi = s.pl[i];
  int cx, cy, cz;
  decode_key(g, key, cx, cy, cz);
  for (int c = 0; c < g.n_diff; ++c) {
    const int nk = key + g.key_diff[c];
    if (nk < 1 || nk > g.key_max) continue;
    const float4 a = rel_to(g, k, pi, cx, cy, cz, nk);
    for (int q = b.cell_start[nk]; q < b.cell_start[nk + 1]; ++q) {
      const int pt = pre_test<DIM>(k, a.x, a.y, a.z, __ldg(&s.pl[q]));
      if (pt == 1) {
        ++cnt;
      } else if (pt < 0) {
        double d[3];
        if (!(dist64<DIM>(s, xp, q, d) > k.h)) ++cnt;
      }
    }
  }
  row_nnz[s.rid[i]] = cnt;
}

template <int DIM>
__global__ void __launch_bounds__(kThreads) asm_fill_kernel(State s, Geometry g, Consts k,
                                                            BinScratch b, int func, double param,
                                                            const int* row_ptr, int* col,
                                                            double* val) {
  const int n = *b.d_n;
  const int i = blockIdx.x * kThreads + threadIdx.x;
  if (i >= n) return;
  const double h2 = k.h * k.h;
  double diag = 0.0;
  if (func == SPH_MAT_PROJECTION) {
    double div, L, lam;
    div_L_lambda<DIM>(s, g, k, b, i, div, L, lam);
    diag = s.type[i] == kFluid ? h2 * L + param * (lam > 0.0 ? lam : 0.0) : h2 * L;
  }
  const int key = s.cell[i];
  double xp[3] = {s.x[0][i], s.x[1][i], DIM == 3 ? s.x[2][i] : 0.0};
  int pos = row_ptr[s.rid[i]];
  const int end = row_ptr[s.rid[i] + 1];
  const float4 pi = s.pl[i];
  int cx, cy, cz;
  decode_key(g, key, cx, cy, cz);
  for (int c = 0; c < g.n_diff; ++c) {
    const int nk = key + g.key_diff[c];
    if (nk < 1 || nk > g.key_max) continue;
    const float4 a = rel_to(g, k, pi, cx, cy, cz, nk);
    for (int q = b.cell_start[nk]; q < b.cell_start[nk + 1]; ++q) {
      const int pt = pre_test<DIM>(k, a.x, a.y, a.z, __ldg(&s.pl[q]));
      if (pt == 0) continue;
      double d[3];
      const double r = dist64<DIM>(s, xp, q, d);
      if (pt < 0 && r > k.h) continue;
      double v;
      if (func == SPH_MAT_KERNEL)
        v = ker_w(k, r);
      else
        v = q == i ? diag : (((2.0 * h2) * k.mass) / k.rho0) * ker_rdw(k, r);
      if (pos < end) {
        col[pos] = s.rid[q];
        val[pos] = v;
      }
      ++pos;
    }
  }
}

// one warp per row: entry e goes to position (number of columns < col[e])
__global__ void __launch_bounds__(kThreads) asm_sort_kernel(int n, const int* row_ptr,
                                                            const int* col_in, const double* val_in,
                                                            int* col_out, double* val_out) {
  const int row = blockIdx.x * (kThreads / 32) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (row >= n) return;
  const int st = row_ptr[row], en = row_ptr[row + 1];
  for (int e = st + lane; e < en; e += 32) {
    const int c = col_in[e];
    int rank = 0;
    for (int f = st; f < en; ++f) rank += col_in[f] < c;
    col_out[st + rank] = c;
    val_out[st + rank] = val_in[e];
  }
}

template <int DIM>
__global__ void __launch_bounds__(kThreads) asm_vector_kernel(State s, Geometry g, Consts k,
                                                              BinScratch b, int func, double* out) {
  const int n = *b.d_n;
  const int i = blockIdx.x * kThreads + threadIdx.x;
  if (i >= n) return;
  double div, L, lam;
  div_L_lambda<DIM>(s, g, k, b, i, div, L, lam);
  // projection_vector: -h^2 p.div / dt
  out[s.rid[i]] = func == SPH_VEC_PROJECTION ? ((-(k.h * k.h)) * div) / k.dt : 0.0;
}

// total of the row counts in 64 bits (the scan is 32-bit)
__global__ void __launch_bounds__(256) count64_kernel(int n, const int* cnt,
                                                      unsigned long long* total) {
  unsigned long long v = 0;
  for (int i = blockIdx.x * 256 + threadIdx.x; i < n; i += gridDim.x * 256) v += (unsigned)cnt[i];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0 && v) atomicAdd(total, v);
}

// ---- CG pieces
__global__ void __launch_bounds__(256) spmv_kernel(int n, const int* row_ptr, const int* col,
                                                   const double* val, const double* x, double* y) {
  const int row = blockIdx.x * 8 + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (row >= n) return;
  double acc = 0.0;
  for (int e = row_ptr[row] + lane; e < row_ptr[row + 1]; e += 32) acc += val[e] * x[col[e]];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if (lane == 0) y[row] = acc;
}

__device__ __forceinline__ double block_sum(double v, double* sh) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if (lane == 0) sh[w] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x == 0)
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) t += sh[i];
  __syncthreads();
  return t;
}

// partial[block] = sum over the block's fixed slice of a[i] * b[i]
__global__ void __launch_bounds__(256) dot_kernel(int n, const double* a, const double* b,
                                                  double* partial) {
  __shared__ double sh[8];
  double v = 0.0;
  for (int i = blockIdx.x * 256 + threadIdx.x; i < n; i += gridDim.x * 256) v += a[i] * b[i];
  const double t = block_sum(v, sh);
  if (threadIdx.x == 0) partial[blockIdx.x] = t;
}

// out[slot] = sum of the partials, in order
__global__ void __launch_bounds__(32) dot_final_kernel(const double* partial, int np, double* out,
                                                       int slot) {
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int i = 0; i < np; ++i) t += partial[i];
    out[slot] = t;
  }
}

// scalars: [0] r.r, [1] p.Ap, [2] r.r new, [3] alpha, [4] beta
__global__ void cg_alpha_kernel(double* sc) { sc[3] = sc[0] / sc[1]; }
__global__ void cg_beta_kernel(double* sc) {
  sc[4] = sc[2] / sc[0];
  sc[0] = sc[2];
}

// x += alpha p; r -= alpha Ap
__global__ void __launch_bounds__(256) cg_update_kernel(int n, const double* sc, double* x,
                                                        double* r, const double* p,
                                                        const double* ap) {
  const int i = blockIdx.x * 256 + threadIdx.x;
  if (i >= n) return;
  const double a = sc[3];
  x[i] += a * p[i];
  r[i] -= a * ap[i];
}

// p = r + beta p
__global__ void __launch_bounds__(256) cg_dir_kernel(int n, const double* sc, const double* r,
                                                     double* p) {
  const int i = blockIdx.x * 256 + threadIdx.x;
  if (i >= n) return;
  p[i] = r[i] + sc[4] * p[i];
}

}  // namespace

struct sph_csr {
  int device = 0;
  int n = 0;
  long long nnz = 0;
  int* row_ptr = nullptr;
  int* col = nullptr;
  double* val = nullptr;
  cudaStream_t stream = nullptr;
};

namespace {

void csr_free(sph_csr* a) {
  if (a->row_ptr) cudaFree(a->row_ptr);
  if (a->col) cudaFree(a->col);
  if (a->val) cudaFree(a->val);
  if (a->stream) cudaStreamDestroy(a->stream);
  delete a;
}

template <int DIM>
cudaError_t assemble_dim(sph_system* s, int func, double param, int* row_nnz, int* row_ptr,
                         int* stmp, int* col_tmp, double* val_tmp, int pass) {
  const LaunchCtx c = system_ctx(s);
  const int blocks = (s->n_host + kThreads - 1) / kThreads;
  mark(c, SPH_KERNEL_SUM, 0);
  if (pass == 0)
    asm_count_kernel<DIM><<<blocks, kThreads, 0, s->stream>>>(s->cur, s->geo, s->k, s->b, row_nnz);
  else
    asm_fill_kernel<DIM><<<blocks, kThreads, 0, s->stream>>>(s->cur, s->geo, s->k, s->b, func,
                                                             param, row_ptr, col_tmp, val_tmp);
  mark(c, SPH_KERNEL_SUM, 1);
  return cudaGetLastError();
}

}  // namespace

extern "C" {

int sph_assemble_matrix(sph_system* s, int func, double param, sph_csr** out) {
  if (!s || !out) return SPH_ERR_ARG;
  *out = nullptr;
  if (func != SPH_MAT_KERNEL && func != SPH_MAT_PROJECTION)
    return system_fail(s, SPH_ERR_ARG, "unknown matrix function");
  if (!s->cells_valid) return system_fail(s, SPH_ERR_STATE, "cell list is stale: call sph_create_cell_list");
  DeviceGuard guard(s->device);
  int n = 0;  // the device-resident count (removals may have lowered it)
  if (cudaMemcpyAsync(&n, s->b.d_n, sizeof(int), cudaMemcpyDeviceToHost, s->stream) != cudaSuccess ||
      cudaStreamSynchronize(s->stream) != cudaSuccess)
    return system_fail(s, SPH_ERR_CUDA, "reading the particle count failed");
  sph_csr* a = new sph_csr();
  a->device = s->device;
  a->n = n;
  const size_t scan_ints = scan_tmp_ints(n + 1) + 64;
  int* row_nnz = nullptr;
  int* stmp = nullptr;
  bool ok = cudaStreamCreateWithFlags(&a->stream, cudaStreamNonBlocking) == cudaSuccess &&
            cudaMalloc(&a->row_ptr, 4 * (size_t)(n + 1)) == cudaSuccess &&
            cudaMalloc(&row_nnz, 4 * (size_t)(n + 1)) == cudaSuccess &&
            cudaMalloc(&stmp, 4 * scan_ints + 512) == cudaSuccess;
  // the 64-bit counter needs 8-byte alignment: its own 256-byte slot
  unsigned long long* total64 =
      stmp ? (unsigned long long*)(((uintptr_t)(stmp + scan_ints) + 255) & ~(uintptr_t)255)
           : nullptr;
  cudaError_t e = cudaSuccess;
  if (ok) {
    e = cudaMemsetAsync(row_nnz + n, 0, sizeof(int), s->stream);
    if (e == cudaSuccess)
      e = s->params.dim == 2 ? assemble_dim<2>(s, func, param, row_nnz, nullptr, nullptr, nullptr, nullptr, 0)
                             : assemble_dim<3>(s, func, param, row_nnz, nullptr, nullptr, nullptr, nullptr, 0);
    unsigned long long t64 = 0;
    if (e == cudaSuccess) e = cudaMemsetAsync(total64, 0, 8, s->stream);
    if (e == cudaSuccess && n > 0) {
      count64_kernel<<<kDotBlocks, 256, 0, s->stream>>>(n, row_nnz, total64);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(&t64, total64, 8, cudaMemcpyDeviceToHost, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    if (e == cudaSuccess && t64 >= 0x7fffffffULL) {
      if (row_nnz) cudaFree(row_nnz);
      cudaFree(stmp);
      csr_free(a);
      return system_fail(s, SPH_ERR_ARG, "the matrix would hold 2^31 or more entries");
    }
    if (e == cudaSuccess) e = launch_scan(system_ctx(s), row_nnz, a->row_ptr, n + 1, stmp);
    a->nnz = (long long)t64;
  }
  int* col_tmp = nullptr;
  double* val_tmp = nullptr;
  if (ok && e == cudaSuccess) {
    const size_t nz = (size_t)(a->nnz > 0 ? a->nnz : 1);
    ok = cudaMalloc(&a->col, 4 * nz) == cudaSuccess && cudaMalloc(&a->val, 8 * nz) == cudaSuccess &&
         cudaMalloc(&col_tmp, 4 * nz) == cudaSuccess && cudaMalloc(&val_tmp, 8 * nz) == cudaSuccess;
    if (ok) {
      e = s->params.dim == 2 ? assemble_dim<2>(s, func, param, nullptr, a->row_ptr, nullptr, col_tmp, val_tmp, 1)
                             : assemble_dim<3>(s, func, param, nullptr, a->row_ptr, nullptr, col_tmp, val_tmp, 1);
      if (e == cudaSuccess && n > 0) {
        asm_sort_kernel<<<(n + (kThreads / 32) - 1) / (kThreads / 32), kThreads, 0, s->stream>>>(
            n, a->row_ptr, col_tmp, val_tmp, a->col, a->val);
        e = cudaGetLastError();
      }
      if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    }
  }
  if (row_nnz) cudaFree(row_nnz);
  if (stmp) cudaFree(stmp);
  if (col_tmp) cudaFree(col_tmp);
  if (val_tmp) cudaFree(val_tmp);
  if (!ok || e != cudaSuccess) {
    cudaGetLastError();
    csr_free(a);
    return system_fail(s, ok ? SPH_ERR_CUDA : SPH_ERR_NOMEM, "matrix assembly failed");
  }
  *out = a;
  return SPH_OK;
}

int sph_assemble_vector(sph_system* s, int func, double* out) {
  if (!s || !out) return SPH_ERR_ARG;
  if (func != SPH_VEC_PROJECTION) return system_fail(s, SPH_ERR_ARG, "unknown vector function");
  if (!s->cells_valid) return system_fail(s, SPH_ERR_STATE, "cell list is stale: call sph_create_cell_list");
  DeviceGuard guard(s->device);
  const int n = s->n_host;
  if (n == 0) return SPH_OK;
  double* d = nullptr;
  if (cudaMalloc(&d, 8 * (size_t)n) != cudaSuccess) {
    cudaGetLastError();
    return system_fail(s, SPH_ERR_NOMEM, "cannot allocate the vector");
  }
  const LaunchCtx c = system_ctx(s);
  mark(c, SPH_KERNEL_SUM, 0);
  const int blocks = (n + kThreads - 1) / kThreads;
  if (s->params.dim == 2)
    asm_vector_kernel<2><<<blocks, kThreads, 0, s->stream>>>(s->cur, s->geo, s->k, s->b, func, d);
  else
    asm_vector_kernel<3><<<blocks, kThreads, 0, s->stream>>>(s->cur, s->geo, s->k, s->b, func, d);
  mark(c, SPH_KERNEL_SUM, 1);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(out, d, 8 * (size_t)n, cudaMemcpyDeviceToHost, s->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
  cudaFree(d);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return system_fail(s, SPH_ERR_CUDA, "vector assembly failed");
  }
  return SPH_OK;
}

int sph_csr_info(const sph_csr* a, int64_t* n, int64_t* nnz) {
  if (!a) return SPH_ERR_ARG;
  if (n) *n = a->n;
  if (nnz) *nnz = a->nnz;
  return SPH_OK;
}

int sph_csr_download(sph_csr* a, int64_t* row_ptr, int32_t* col, double* val) {
  if (!a) return SPH_ERR_ARG;
  DeviceGuard guard(a->device);
  std::vector<int> rp((size_t)a->n + 1);
  cudaError_t e = cudaMemcpy(rp.data(), a->row_ptr, 4 * rp.size(), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && col && a->nnz)
    e = cudaMemcpy(col, a->col, 4 * (size_t)a->nnz, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && val && a->nnz)
    e = cudaMemcpy(val, a->val, 8 * (size_t)a->nnz, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return SPH_ERR_CUDA;
  }
  if (row_ptr)
    for (size_t i = 0; i < rp.size(); ++i) row_ptr[i] = rp[i];
  return SPH_OK;
}

int sph_csr_destroy(sph_csr* a) {
  if (!a) return SPH_ERR_ARG;
  DeviceGuard guard(a->device);
  cudaStreamSynchronize(a->stream);
  csr_free(a);
  return SPH_OK;
}

int sph_cg(sph_csr* a, const double* b, double* x, double reltol, int32_t maxiter,
           int32_t* iters, double* resid) {
  if (!a || !b || !x || !(reltol >= 0.0)) return SPH_ERR_ARG;
  DeviceGuard guard(a->device);
  const int n = a->n;
  if (maxiter < 0) maxiter = n;  // IterativeSolvers' default: size(A, 2)
  if (n == 0) {
    if (iters) *iters = 0;
    if (resid) *resid = 0.0;
    return SPH_OK;
  }
  double* w = nullptr;  // x, r, p, Ap, b, partials, scalars
  const size_t N = (size_t)n;
  if (cudaMalloc(&w, 8 * (5 * N + kDotBlocks + 8)) != cudaSuccess) {
    cudaGetLastError();
    return SPH_ERR_NOMEM;
  }
  double *dx = w, *dr = w + N, *dp = w + 2 * N, *dap = w + 3 * N, *db = w + 4 * N;
  double* part = w + 5 * N;
  double* sc = part + kDotBlocks;
  cudaStream_t st = a->stream;
  const int eb = (n + 255) / 256, rb = (n + 7) / 8;
  auto dot = [&](const double* u, const double* v, int slot) {
    dot_kernel<<<kDotBlocks, 256, 0, st>>>(n, u, v, part);
    dot_final_kernel<<<1, 32, 0, st>>>(part, kDotBlocks, sc, slot);
  };
  double bb = 0.0, rr = 0.0;
  cudaError_t e = cudaMemcpyAsync(db, b, 8 * N, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(dx, 0, 8 * N, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dr, db, 8 * N, cudaMemcpyDeviceToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dp, db, 8 * N, cudaMemcpyDeviceToDevice, st);
  if (e == cudaSuccess) {
    dot(db, db, 0);
    e = cudaMemcpyAsync(&bb, sc, 8, cudaMemcpyDeviceToHost, st);
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  const double tol = reltol * std::sqrt(bb);
  rr = bb;
  int it = 0;
  while (e == cudaSuccess && !(std::sqrt(rr) <= tol) && it < maxiter) {
    spmv_kernel<<<rb, 256, 0, st>>>(n, a->row_ptr, a->col, a->val, dp, dap);
    dot(dp, dap, 1);
    cg_alpha_kernel<<<1, 1, 0, st>>>(sc);
    cg_update_kernel<<<eb, 256, 0, st>>>(n, sc, dx, dr, dp, dap);
    dot(dr, dr, 2);
    cg_beta_kernel<<<1, 1, 0, st>>>(sc);
    cg_dir_kernel<<<eb, 256, 0, st>>>(n, sc, dr, dp);
    e = cudaMemcpyAsync(&rr, sc, 8, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    ++it;
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(x, dx, 8 * N, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cudaFree(w);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return SPH_ERR_CUDA;
  }
  if (iters) *iters = it;
  if (resid) *resid = std::sqrt(rr);
  return SPH_OK;
}

}  // extern "C"
