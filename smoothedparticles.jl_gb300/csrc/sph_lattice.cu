// sph_lattice.cu -- device-side particle generation: covering(grid, shape) of
// SmoothedParticles.jl for the shapes of the dam-break inputs.
//
//   * square / cubic grid: points i*dr for integer i from floor(lo/dr) to
//     ceil(hi/dr) of the shape's bounding box, i outer, then j, then k
//     (src/grids.jl:52-66, :128-144);
//   * Box / Rectangle: lo[d] <= x[d] <= hi[d] for every d (src/geometry.jl:24-43);
//   * BoundaryLayer(box, grid, width): bounding box grown by width, a point
//     outside the box with some lattice offset dx, |dx| <= width, such that
//     x + dx is inside (src/geometry.jl:198-234), optionally restricted by a
//     Specification predicate x[axis] < keep (src/geometry.jl:179-196).
//
// Every point of the bounding box is one thread: flag, exclusive scan (the
// order-preserving compaction), write.  Compiled with --fmad=false; the
// arithmetic is i * dr and the box comparisons, so the points are the ones the
// host restatement (sphgpu/geometry.py) produces, bit for bit.
#include <cmath>

#include "sph_launch.h"
#include "sphgpu.h"

namespace sphgpu {

namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ bool in_box(const LatticeShape& s, const double x[3]) {
  bool in = true;
#pragma unroll
  for (int d = 0; d < 3; ++d) in = in && (s.lo[d] <= x[d]) && (x[d] <= s.hi[d]);
  return in;
}

__device__ __forceinline__ void point(const LatticeShape& s, long long idx, double x[3]) {
  const long long k = idx % s.n[2];
  const long long t = idx / s.n[2];
  const long long j = t % s.n[1];
  const long long i = t / s.n[1];
  x[0] = (double)(s.i0[0] + i) * s.dr;
  x[1] = (double)(s.i0[1] + j) * s.dr;
  x[2] = s.dim == 3 ? (double)(s.i0[2] + k) * s.dr : 0.0;
}

__device__ __forceinline__ bool member(const LatticeShape& s, const double* offs, const double x[3]) {
  if (s.kind == SPH_SHAPE_BOX) return in_box(s, x);
  if (in_box(s, x)) return false;
  if (s.keep_axis >= 0 && !(x[s.keep_axis] < s.keep_max)) return false;
  for (int o = 0; o < s.n_off; ++o) {
    const double y[3] = {x[0] + offs[3 * o], x[1] + offs[3 * o + 1], x[2] + offs[3 * o + 2]};
    if (in_box(s, y)) return true;
  }
  return false;
}

__global__ void __launch_bounds__(kThreads) lattice_flags_kernel(LatticeShape s, const double* offs,
                                                                 int* flags, long long total) {
  const long long idx = (long long)blockIdx.x * kThreads + threadIdx.x;
  if (idx >= total) return;
  double x[3];
  point(s, idx, x);
  flags[idx] = member(s, offs, x) ? 1 : 0;
}

__global__ void __launch_bounds__(kThreads) lattice_write_kernel(LatticeShape s, const int* flags,
                                                                 const int* pos, long long total,
                                                                 double* xout, int* tout, int base) {
  const long long idx = (long long)blockIdx.x * kThreads + threadIdx.x;
  if (idx >= total || !flags[idx]) return;
  double x[3];
  point(s, idx, x);
  const long long p = (long long)base + pos[idx];
  xout[3 * p] = x[0];
  xout[3 * p + 1] = x[1];
  xout[3 * p + 2] = x[2];
  tout[p] = s.type;
}

// Int64(floor(lo / dr)) : Int64(ceil(hi / dr))
bool axis_range(double lo, double hi, double dr, long long& i0, long long& n) {
  const double a = std::floor(lo / dr);
  const double b = std::ceil(hi / dr);
  if (!(a >= -4.0e15 && b <= 4.0e15) || b < a) return false;
  i0 = (long long)a;
  n = (long long)b - i0 + 1;
  return true;
}

}  // namespace

int lattice_prepare(const sph_shape& in, int dim, LatticeShape& out, std::vector<double>& offs) {
  if (!(in.dr > 0.0) || (in.kind != SPH_SHAPE_BOX && in.kind != SPH_SHAPE_LAYER) ||
      (in.type != SPH_FLUID && in.type != SPH_WALL) || in.keep_axis < -1 || in.keep_axis >= dim)
    return SPH_ERR_ARG;
  for (int d = 0; d < 3; ++d)
    if (!(in.lo[d] <= in.hi[d])) return SPH_ERR_ARG;
  if (dim == 2 && (in.lo[2] != 0.0 || in.hi[2] != 0.0)) return SPH_ERR_ARG;
  out = LatticeShape{};
  out.kind = in.kind;
  out.type = in.type;
  out.dim = dim;
  out.keep_axis = in.kind == SPH_SHAPE_LAYER ? in.keep_axis : -1;
  out.keep_max = in.keep_max;
  out.dr = in.dr;
  double blo[3], bhi[3];
  for (int d = 0; d < 3; ++d) {
    out.lo[d] = in.lo[d];
    out.hi[d] = in.hi[d];
    const double w = in.kind == SPH_SHAPE_LAYER ? in.width : 0.0;
    blo[d] = (dim == 2 && d == 2) ? 0.0 : in.lo[d] - w;
    bhi[d] = (dim == 2 && d == 2) ? 0.0 : in.hi[d] + w;
  }
  for (int d = 0; d < 3; ++d) {
    if (dim == 2 && d == 2) {
      out.i0[2] = 0;
      out.n[2] = 1;
    } else if (!axis_range(blo[d], bhi[d], in.dr, out.i0[d], out.n[d])) {
      return SPH_ERR_ARG;
    }
  }
  offs.clear();
  if (in.kind == SPH_SHAPE_LAYER) {
    // covering(grid, Ball(0, 0, 0, width)): (x1^2 + x2^2) + x3^2 <= width^2
    if (!(in.width >= 0.0)) return SPH_ERR_ARG;
    const double w = in.width;
    long long b0[3], bn[3];
    for (int d = 0; d < 3; ++d) {
      if (dim == 2 && d == 2) {
        b0[2] = 0;
        bn[2] = 1;
      } else if (!axis_range(-w, w, in.dr, b0[d], bn[d])) {
        return SPH_ERR_ARG;
      }
    }
    for (long long i = 0; i < bn[0]; ++i)
      for (long long j = 0; j < bn[1]; ++j)
        for (long long k = 0; k < bn[2]; ++k) {
          const double x = (double)(b0[0] + i) * in.dr;
          const double y = (double)(b0[1] + j) * in.dr;
          const double z = dim == 3 ? (double)(b0[2] + k) * in.dr : 0.0;
          const double s = (x * x + y * y) + z * z;
          if (s <= w * w) {
            offs.push_back(x);
            offs.push_back(y);
            offs.push_back(z);
          }
        }
  }
  out.n_off = (int)(offs.size() / 3);
  return SPH_OK;
}

long long lattice_points(const LatticeShape& s) { return s.n[0] * s.n[1] * s.n[2]; }

cudaError_t launch_lattice_flags(const LaunchCtx& c, const LatticeShape& s, const double* offs,
                                 int* flags) {
  const long long total = lattice_points(s);
  if (total <= 0) return cudaSuccess;
  mark(c, SPH_KERNEL_IO, 0);
  lattice_flags_kernel<<<(unsigned)((total + kThreads - 1) / kThreads), kThreads, 0, c.stream>>>(
      s, offs, flags, total);
  mark(c, SPH_KERNEL_IO, 1);
  return cudaGetLastError();
}

cudaError_t launch_lattice_write(const LaunchCtx& c, const LatticeShape& s, const int* flags,
                                 const int* pos, double* x, int* type, int base) {
  const long long total = lattice_points(s);
  if (total <= 0) return cudaSuccess;
  mark(c, SPH_KERNEL_IO, 0);
  lattice_write_kernel<<<(unsigned)((total + kThreads - 1) / kThreads), kThreads, 0, c.stream>>>(
      s, flags, pos, total, x, type, base);
  mark(c, SPH_KERNEL_IO, 1);
  return cudaGetLastError();
}

}  // namespace sphgpu
