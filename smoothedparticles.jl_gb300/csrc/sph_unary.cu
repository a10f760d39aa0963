// sph_unary.cu -- apply_unary! (core.jl:138-142) with the built-in unary
// operators, and the particle-field transfer between the cell-ordered device
// arrays and reference-ordered host buffers (ParticleField, structs.jl:118-125).
//
// Built with --fmad=false (same expression rounding as the CPU restatement).
// All kernels are HBM-bound element-wise passes, one thread per particle.
#include "sph_launch.h"
#include "sphgpu.h"

namespace sphgpu {

namespace {

constexpr int kThreads = 256;

template <int DIM>
__device__ __forceinline__ void unary_body(const State& s, const Consts& k, const BinScratch& b,
                                           int op, int blk) {
  const int n = *b.d_n;
  const int i = blk * kThreads + threadIdx.x;
  if (i >= n) return;
  const bool fluid = s.type[i] == kFluid;
  switch (op) {
    case SPH_OP_RESET_RHO:
      s.rho[i] = 0.0;
      break;
    case SPH_OP_RESET_RHO_REF:
      s.rho_ref[i] = 0.0;
      break;
    case SPH_OP_RESET_A:
#pragma unroll
      for (int d = 0; d < DIM; ++d) {
        s.a[d][i] = 0.0;
        s.xs[d][i] = 0.0;
      }
      break;
    case SPH_OP_EOS:  // the system's equation of state (eos_eval)
      if (fluid) {
        double P, Pr;
        eos_eval(k, s.rho[i], s.rho_ref[i], P, Pr);
        s.P[i] = P;
        s.Pr[i] = Pr;
      } else {
        s.P[i] = 0.0;
        s.Pr[i] = 0.0;
      }
      break;
    case SPH_OP_KICK:  // accelerate! (collapse_symplectic.jl:139-143)
      if (fluid) {
#pragma unroll
        for (int d = 0; d < DIM; ++d) s.v[d][i] = s.v[d][i] + k.hdt * (s.a[d][i] + k.g[d]);
      }
      break;
    case SPH_OP_DRIFT:  // move! (collapse_symplectic.jl:133-137) with XSPH
      if (fluid) {
#pragma unroll
        for (int d = 0; d < DIM; ++d)
          s.x[d][i] = s.x[d][i] + k.dt * (s.v[d][i] + k.eps_xsph * s.xs[d][i]);
      }
      break;
    case SPH_OP_HYDROSTATIC:
      if (fluid) {
        const double y = s.x[k.vaxis][i];
        const double u = (k.rho0 * k.gmag * (k.col_height - y)) / k.B;
        const double cc = 1.0 + u;
        double f = 1.0 + u / 7.0;
        for (int it = 0; it < 6; ++it) {  // Newton iterations for f^7 = 1 + u
          const double f2 = f * f;
          const double f3 = f2 * f;
          const double f6 = f3 * f3;
          const double f7 = f6 * f;
          f = f - (f7 - cc) / (7.0 * f6);
        }
        s.rho_ref[i] = s.rho_ref[i] / f;
      }
      break;
    default:
      break;
  }
}

template <int DIM>
__global__ void __launch_bounds__(kThreads) unary_kernel(State s, Consts k, BinScratch b, int op) {
  unary_body<DIM>(s, k, b, op, blockIdx.x);
}

// fused batches: block i works on map[i] = (member, block of that member)
template <int DIM>
__global__ void __launch_bounds__(kThreads) unary_fused_kernel(const MemberArgs* __restrict__ margs,
                                                               const int2* __restrict__ map, int op) {
  const int2 e = map[blockIdx.x];
  const MemberArgs& m = margs[e.x];
  unary_body<DIM>(m.cur, m.k, m.b, op, e.y);
}

template <int DIM>
__global__ void __launch_bounds__(kThreads) upload_kernel(State s, BinScratch b, int n,
                                                          const double* x, const double* v,
                                                          const double* rho,
                                                          const double* rho_ref,
                                                          const int* type) {
  const int i = blockIdx.x * kThreads + threadIdx.x;
  if (i == 0) *b.d_n = n;
  if (i >= n) return;
#pragma unroll
  for (int d = 0; d < DIM; ++d) {
    s.x[d][i] = x[3 * i + d];
    s.v[d][i] = v ? v[3 * i + d] : 0.0;
    s.a[d][i] = 0.0;
    s.xs[d][i] = 0.0;
  }
  s.rho[i] = rho ? rho[i] : 0.0;
  s.rho_ref[i] = rho_ref ? rho_ref[i] : 0.0;
  s.P[i] = 0.0;
  s.Pr[i] = 0.0;
  const int t = type ? type[i] : kFluid;
  s.type[i] = t;
  s.rid[i] = i;
  s.oid[i] = i;
  s.cell[i] = 0;
  s.pl[i] = make_float4(0.f, 0.f, 0.f, __int_as_float(t));
  b.inv_rid[i] = i;
  b.ident[i] = i;
  b.flag_by_rid[i] = 0;
}

// dir 0: state (cell order) -> staging (reference order); dir 1: the reverse.
template <int DIM>
__global__ void __launch_bounds__(kThreads) field_kernel(State s, BinScratch b, int field,
                                                         int dir, void* staging, int eos,
                                                         double rho0sq) {
  const int n = *b.d_n;
  const int i = blockIdx.x * kThreads + threadIdx.x;
  if (i >= n) return;
  const int r = s.rid[i];
  double* const* vec = nullptr;
  double* sc = nullptr;
  switch (field) {
    case SPH_FIELD_X: vec = s.x; break;
    case SPH_FIELD_V: vec = s.v; break;
    case SPH_FIELD_A: vec = s.a; break;
    case SPH_FIELD_XSPH: vec = s.xs; break;
    case SPH_FIELD_RHO: sc = s.rho; break;
    case SPH_FIELD_RHO_REF: sc = s.rho_ref; break;
    case SPH_FIELD_P: sc = s.P; break;
    default: break;
  }
  if (vec) {
    double* st = (double*)staging;
    if (dir == 0) {
#pragma unroll
      for (int d = 0; d < 3; ++d) st[3 * r + d] = d < DIM ? vec[d][i] : 0.0;
    } else {
#pragma unroll
      for (int d = 0; d < DIM; ++d) vec[d][i] = st[3 * r + d];
    }
  } else if (sc) {
    double* st = (double*)staging;
    if (dir == 0) {
      st[r] = sc[i];
    } else {
      sc[i] = st[r];
      if (field == SPH_FIELD_P)
        s.Pr[i] = s.type[i] != kFluid ? 0.0
                  : eos == 1         ? st[r] / rho0sq
                                     : st[r] / (s.rho[i] * s.rho[i]);
    }
  } else if (field == SPH_FIELD_TYPE) {
    int* st = (int*)staging;
    if (dir == 0) {
      st[r] = s.type[i];
    } else {
      s.type[i] = st[r];
      s.pl[i].w = __int_as_float(st[r]);
    }
  } else if (field == SPH_FIELD_OID) {
    ((long long*)staging)[r] = s.oid[i];
  } else if (field == SPH_FIELD_KEY) {
    ((long long*)staging)[r] = s.cell[i];
  }
}

}  // namespace

cudaError_t launch_unary(const LaunchCtx& c, const State& s, const Consts& k,
                         const BinScratch& b, int cap, int op) {
  if (cap <= 0) return cudaSuccess;
  const int blocks = (cap + kThreads - 1) / kThreads;
  mark(c, SPH_KERNEL_UNARY, 0);
  if (k.dim == 2)
    unary_kernel<2><<<blocks, kThreads, 0, c.stream>>>(s, k, b, op);
  else
    unary_kernel<3><<<blocks, kThreads, 0, c.stream>>>(s, k, b, op);
  mark(c, SPH_KERNEL_UNARY, 1);
  return cudaGetLastError();
}

cudaError_t launch_upload(const LaunchCtx& c, const State& s, const Consts& k,
                          const BinScratch& b, int n, const double* x, const double* v,
                          const double* rho, const double* rho_ref, const int* type) {
  const int blocks = n > 0 ? (n + kThreads - 1) / kThreads : 1;
  mark(c, SPH_KERNEL_IO, 0);
  if (k.dim == 2)
    upload_kernel<2><<<blocks, kThreads, 0, c.stream>>>(s, b, n, x, v, rho, rho_ref, type);
  else
    upload_kernel<3><<<blocks, kThreads, 0, c.stream>>>(s, b, n, x, v, rho, rho_ref, type);
  mark(c, SPH_KERNEL_IO, 1);
  return cudaGetLastError();
}

cudaError_t launch_fused_unary(const LaunchCtx& c, const FusedBatch& fb, int p, int op) {
  mark(c, SPH_KERNEL_UNARY, 0);
  const unsigned grid = (unsigned)fb.blocks[kShapeParticles];
  if (fb.dim == 2)
    unary_fused_kernel<2><<<grid, kThreads, 0, c.stream>>>(fb.args[p], fb.map[kShapeParticles], op);
  else
    unary_fused_kernel<3><<<grid, kThreads, 0, c.stream>>>(fb.args[p], fb.map[kShapeParticles], op);
  mark(c, SPH_KERNEL_UNARY, 1);
  return cudaGetLastError();
}

cudaError_t launch_field(const LaunchCtx& c, const State& s, const Consts& k,
                         const BinScratch& b, int cap, int field, int dir, void* staging) {
  if (cap <= 0) return cudaSuccess;
  const int blocks = (cap + kThreads - 1) / kThreads;
  mark(c, SPH_KERNEL_IO, 0);
  if (k.dim == 2)
    field_kernel<2><<<blocks, kThreads, 0, c.stream>>>(s, b, field, dir, staging, k.eos, k.rho0sq);
  else
    field_kernel<3><<<blocks, kThreads, 0, c.stream>>>(s, b, field, dir, staging, k.eos, k.rho0sq);
  mark(c, SPH_KERNEL_IO, 1);
  return cudaGetLastError();
}

}  // namespace sphgpu
