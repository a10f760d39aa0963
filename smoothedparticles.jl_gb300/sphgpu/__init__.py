"""sphgpu -- host-side mirror of SmoothedParticles.jl's cell-list / pair-loop
surface over the GB300 C ABI (include/sphgpu.h).

Names follow the reference (src/SmoothedParticles.jl:9-72) with Julia's ``!``
dropped: ``ParticleSystem`` (structs.jl:57), ``create_cell_list``
(core.jl:51), ``apply`` (core.jl:151), ``apply_unary`` (core.jl:138),
``apply_binary`` (core.jl:125), ``sum`` (core.jl:240, :271) and
``ParticleField`` (structs.jl:118).  Operators are the built-in ones below;
arbitrary closures have no device counterpart and nothing runs on the CPU.
Errors raise ``SphError`` (the reference throws Julia exceptions).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib as L
from ._lib import (SPH_FLUID as FLUID, SPH_WALL as WALL, SPH_PREC_FP64 as FP64,
                   SPH_PREC_MIXED as MIXED)

__all__ = ["ParticleSystem", "ParticleField", "create_cell_list", "apply", "apply_unary",
           "apply_binary", "sum", "SphError", "Operator", "SumFunction", "FLUID", "WALL",
           "FP64", "MIXED", "find_rho", "find_rho0", "internal_force", "find_pressure",
           "reset_rho", "reset_rho0", "reset_a", "accelerate", "move", "hydrostatic",
           "DENSITY", "KERNEL", "PRESSURE", "SHEPARD", "wall_pressure", "Batch", "pipe_peak", "arith_check",
           "memory_estimate", "shape_count", "assemble_matrix", "assemble_vector", "CsrMatrix",
           "MAT_KERNEL", "MAT_PROJECTION", "VEC_PROJECTION"]


class SphError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"sphgpu error {code}: {msg}")
        self.code = code


@dataclass(frozen=True)
class Operator:
    """A built-in operator; ``binary`` mirrors hasmethod(op!, (T, T, Float64))."""
    name: str
    op: int
    binary: bool


@dataclass(frozen=True)
class SumFunction:
    name: str
    func: int


# pair operators (the examples' find_rho!, find_rho0!, internal_force!)
find_rho = Operator("find_rho!", L.SPH_OP_DENSITY, True)
find_rho0 = Operator("find_rho0!", L.SPH_OP_DENSITY_REF, True)
internal_force = Operator("internal_force!", L.SPH_OP_FORCE, True)
wall_pressure = Operator("wall_pressure!", L.SPH_OP_WALL_PRESSURE, True)
# unary operators
find_pressure = Operator("find_pressure!", L.SPH_OP_EOS, False)
reset_rho = Operator("reset_rho!", L.SPH_OP_RESET_RHO, False)
reset_rho0 = Operator("reset_rho0!", L.SPH_OP_RESET_RHO_REF, False)
reset_a = Operator("reset_a!", L.SPH_OP_RESET_A, False)
accelerate = Operator("accelerate!", L.SPH_OP_KICK, False)
move = Operator("move!", L.SPH_OP_DRIFT, False)
hydrostatic = Operator("hydrostatic!", L.SPH_OP_HYDROSTATIC, False)
_BY_ID = {o.op: o for o in (find_rho, find_rho0, internal_force, wall_pressure, find_pressure,
                            reset_rho, reset_rho0, reset_a, accelerate, move, hydrostatic)}


def op_by_id(op: int) -> Operator:
    """The built-in operator with the C ABI's id ``op`` (SPH_OP_*)."""
    return _BY_ID[int(op)]


# functions for sum()
DENSITY = SumFunction("density", L.SPH_SUM_DENSITY)
KERNEL = SumFunction("kernel", L.SPH_SUM_KERNEL)
PRESSURE = SumFunction("pressure", L.SPH_SUM_PRESSURE)
SHEPARD = SumFunction("shepard", L.SPH_SUM_SHEPARD)

_FIELDS = {"x": L.SPH_FIELD_X, "v": L.SPH_FIELD_V, "a": L.SPH_FIELD_A,
           "xsph": L.SPH_FIELD_XSPH, "rho": L.SPH_FIELD_RHO, "rho0": L.SPH_FIELD_RHO_REF,
           "rho_ref": L.SPH_FIELD_RHO_REF, "P": L.SPH_FIELD_P, "type": L.SPH_FIELD_TYPE,
           "oid": L.SPH_FIELD_OID, "key": L.SPH_FIELD_KEY}
_VECTOR = {L.SPH_FIELD_X, L.SPH_FIELD_V, L.SPH_FIELD_A, L.SPH_FIELD_XSPH}


def _ptr(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


class ParticleSystem:
    """ParticleSystem(T, domain, h) (structs.jl:57-92) on one GPU.

    ``params`` holds the domain bounding box, the neighbour radius ``h`` (the
    kernel support) and the physical constants of the built-in operators.
    """

    def __init__(self, params: dict, precision: int = FP64, device: int = 0):
        self._lib = L.load()
        self.params = dict(params)
        self.precision = precision
        p = L.make_params(L.sph_params, params, precision)
        h = C.c_void_p()
        rc = self._lib.sph_create(C.byref(p), int(device), C.byref(h))
        if rc != 0:
            raise SphError(rc, "sph_create failed (invalid parameters or no CUDA device)")
        self._h = h
        self.dim = int(params["dim"])

    # -- lifetime
    def close(self):
        if getattr(self, "_h", None):
            self._lib.sph_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _check(self, rc: int):
        if rc != 0:
            msg = self._lib.sph_last_error(self._h)
            raise SphError(rc, msg.decode() if msg else "")

    # -- geometry and particles
    def geometry(self):
        kp = (C.c_int64 * 3)()
        kl = (C.c_int64 * 3)()
        km = C.c_int64()
        kd = (C.c_int64 * 27)()
        nd = C.c_int32()
        self._check(self._lib.sph_geometry(self._h, kp, kl, C.byref(km), kd, C.byref(nd)))
        return dict(key_phase=tuple(kp), key_lim=tuple(kl), key_max=km.value,
                    key_diff=list(kd)[: nd.value])

    def upload(self, x, v=None, rho=None, rho_ref=None, type=None):
        """generate_particles! (grids.jl:253-258): replaces the particle set."""
        x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1, 3)
        n = x.shape[0]
        v = None if v is None else np.ascontiguousarray(v, dtype=np.float64).reshape(n, 3)
        rho = None if rho is None else np.ascontiguousarray(rho, dtype=np.float64).reshape(n)
        rr = None if rho_ref is None else np.ascontiguousarray(rho_ref, dtype=np.float64).reshape(n)
        t = None if type is None else np.ascontiguousarray(type, dtype=np.int32).reshape(n)
        self._keep = (x, v, rho, rr, t)
        self._check(self._lib.sph_upload(self._h, n, _ptr(x), _ptr(v), _ptr(rho), _ptr(rr), _ptr(t)))
        self._keep = None

    def generate(self, shapes) -> int:
        """generate_particles! on the device (grids.jl:253-258): replaces the
        particle set by the lattice points of ``shapes`` (dicts as produced by
        ``geometry.dam_break_shapes``), in order; returns the particle count."""
        arr = L.make_shapes(shapes)
        n = C.c_int64()
        self._check(self._lib.sph_generate(self._h, arr, len(shapes), C.byref(n)))
        return n.value

    @property
    def n(self) -> int:
        c = C.c_int64()
        self._check(self._lib.sph_num_particles(self._h, C.byref(c)))
        return c.value

    def get(self, name: str, out: np.ndarray | None = None) -> np.ndarray:
        """Whole field in reference order; ``out`` (e.g. a pinned host array of
        the right shape and dtype) receives the data without an extra copy."""
        f = _FIELDS[name]
        n = self.n
        if f in _VECTOR:
            shape, dt = (n, 3), np.float64
        elif f == L.SPH_FIELD_TYPE:
            shape, dt = (n,), np.int32
        elif f in (L.SPH_FIELD_OID, L.SPH_FIELD_KEY):
            shape, dt = (n,), np.int64
        else:
            shape, dt = (n,), np.float64
        if out is None:
            out = np.empty(shape, dt)
        elif out.shape != shape or out.dtype != dt or not out.flags.c_contiguous:
            raise ValueError(f"out must be a C-contiguous {dt.__name__} array of shape {shape}")
        if n:
            self._check(self._lib.sph_get_field(self._h, f, _ptr(out)))
        return out

    def set(self, name: str, values):
        f = _FIELDS[name]
        n = self.n
        if f in _VECTOR:
            a = np.ascontiguousarray(values, dtype=np.float64).reshape(n, 3)
        elif f == L.SPH_FIELD_TYPE:
            a = np.ascontiguousarray(values, dtype=np.int32).reshape(n)
        else:
            a = np.ascontiguousarray(values, dtype=np.float64).reshape(n)
        if n:
            self._check(self._lib.sph_set_field(self._h, f, _ptr(a)))

    # -- the per-step path
    def create_cell_list(self):
        self._check(self._lib.sph_create_cell_list(self._h))

    def apply(self, op: Operator, self_term: bool = False):
        self._check(self._lib.sph_apply(self._h, op.op, 1 if self_term else 0))

    def apply_unary(self, op: Operator):
        self._check(self._lib.sph_apply_unary(self._h, op.op))

    def sum_points(self, func: SumFunction, x) -> np.ndarray:
        x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1, 3)
        out = np.empty(x.shape[0], np.float64)
        self._check(self._lib.sph_sum_point(self._h, func.func, x.shape[0], _ptr(x), _ptr(out)))
        return out

    def sum_particles(self, func: SumFunction, index) -> np.ndarray:
        idx = np.ascontiguousarray(index, dtype=np.int64).reshape(-1)
        out = np.empty(idx.shape[0], np.float64)
        self._check(self._lib.sph_sum_particle(self._h, func.func, idx.shape[0], _ptr(idx), _ptr(out)))
        return out

    def step(self, nsteps: int = 1):
        """verlet_step! (collapse_symplectic.jl:170-180), nsteps times; four or more
        steps per call (with per-kernel timing off) replay a captured two-step
        CUDA graph of this system, with the same results."""
        self._check(self._lib.sph_step(self._h, int(nsteps)))

    def step_io(self, inputs: dict, outputs: dict) -> dict:
        """One step with host input and output (sph_step_io): the arrays of
        ``inputs`` (field name -> array) are set, one step is taken, and the
        fields named in ``outputs`` are read into its arrays (C-contiguous, of
        the dtype and shape ``get`` returns for the count before the step;
        with removals only the leading rows are written).  Reads into pinned
        arrays overlap the rest of the step.  Returns ``outputs``."""
        n = self.n
        ins = []
        for name, vals in inputs.items():
            f = _FIELDS[name]
            if f in _VECTOR:
                a = np.ascontiguousarray(vals, dtype=np.float64).reshape(n, 3)
            elif f == L.SPH_FIELD_TYPE:
                a = np.ascontiguousarray(vals, dtype=np.int32).reshape(n)
            else:
                a = np.ascontiguousarray(vals, dtype=np.float64).reshape(n)
            ins.append((f, a))
        outs = []
        for name, arr in outputs.items():
            f = _FIELDS[name]
            if f in _VECTOR:
                shape, dt = (n, 3), np.float64
            elif f == L.SPH_FIELD_TYPE:
                shape, dt = (n,), np.int32
            elif f in (L.SPH_FIELD_OID, L.SPH_FIELD_KEY):
                shape, dt = (n,), np.int64
            else:
                shape, dt = (n,), np.float64
            if arr.shape != shape or arr.dtype != dt or not arr.flags.c_contiguous:
                raise ValueError(f"{name}: a C-contiguous {dt.__name__} array of shape {shape}")
            outs.append((f, arr))
        fi = (C.c_int32 * max(len(ins), 1))(*[f for f, _ in ins])
        pi = (C.c_void_p * max(len(ins), 1))(*[a.ctypes.data for _, a in ins])
        fo = (C.c_int32 * max(len(outs), 1))(*[f for f, _ in outs])
        po = (C.c_void_p * max(len(outs), 1))(*[a.ctypes.data for _, a in outs])
        self._check(self._lib.sph_step_io(self._h, len(ins), fi, pi, len(outs), fo, po))
        return outputs

    def init_state(self):
        """The dam-break initialisation (collapse_symplectic.jl:186-191 + hydrostatic)."""
        self._check(self._lib.sph_init_state(self._h))

    # -- accounting and diagnostics
    def pair_count(self, reset: bool = False) -> int:
        c = C.c_uint64()
        self._check(self._lib.sph_pair_count(self._h, C.byref(c), 1 if reset else 0))
        return c.value

    def synchronize(self):
        self._check(self._lib.sph_synchronize(self._h))

    def stream(self) -> int:
        p = C.c_void_p()
        self._check(self._lib.sph_stream(self._h, C.byref(p)))
        return p.value or 0

    def debug_pairs(self) -> np.ndarray:
        cnt = C.c_int64()
        self._check(self._lib.sph_debug_pairs(self._h, None, 0, C.byref(cnt)))
        out = np.empty((cnt.value, 2), np.int64)
        if cnt.value:
            self._check(self._lib.sph_debug_pairs(self._h, _ptr(out), cnt.value, C.byref(cnt)))
        return out

    def debug_hits(self) -> np.ndarray:
        """The (p, q) pairs the last density pass stored for the force pass
        (FP64 rows or mixed hit masks), fluid targets, reference order."""
        cnt = C.c_int64()
        self._check(self._lib.sph_debug_hits(self._h, None, 0, C.byref(cnt)))
        out = np.empty((cnt.value, 2), np.int64)
        if cnt.value:
            self._check(self._lib.sph_debug_hits(self._h, _ptr(out), cnt.value, C.byref(cnt)))
        return out

    def set_profiling(self, on: bool = True):
        self._check(self._lib.sph_set_profiling(self._h, 1 if on else 0))

    def kernel_stats(self) -> dict:
        out = {}
        for k, name in enumerate(L.KERNEL_NAMES):
            ms = C.c_double()
            nl = C.c_int64()
            self._check(self._lib.sph_kernel_stats(self._h, k, C.byref(ms), C.byref(nl)))
            out[name] = (ms.value, nl.value)
        return out

    def reset_kernel_stats(self):
        self._check(self._lib.sph_reset_kernel_stats(self._h))

    def launch_count(self) -> int:
        c = C.c_int64()
        self._check(self._lib.sph_launch_count(self._h, C.byref(c)))
        return c.value

    def memory_usage(self) -> int:
        """Device bytes this system holds now."""
        b = C.c_uint64()
        self._check(self._lib.sph_memory_usage(self._h, C.byref(b)))
        return b.value

    def idle(self) -> bool:
        """True when all queued work of this system has finished (never waits)."""
        i = C.c_int()
        self._check(self._lib.sph_query(self._h, C.byref(i)))
        return bool(i.value)

    def set_tuning(self, warps_per_block: int):
        """Warps per block of the pair passes (2, 4 or 8); results do not change."""
        self._check(self._lib.sph_set_tuning(self._h, int(warps_per_block)))

    def tuning(self) -> int:
        w = C.c_int()
        self._check(self._lib.sph_get_tuning(self._h, C.byref(w)))
        return w.value

    def set_chunk_threads(self, threads: int):
        """Threads per cell chunk of the mixed pair passes (32, 64 or 128);
        mixed results change at the FP32 level, reproducibly per setting."""
        self._check(self._lib.sph_set_chunk_threads(self._h, int(threads)))

    def chunk_threads(self) -> int:
        t = C.c_int()
        self._check(self._lib.sph_get_chunk_threads(self._h, C.byref(t)))
        return t.value

    def pair_stats(self, reset: bool = False) -> dict:
        """Hits per category: density, wall (pressure pass), force_fluid,
        force_wall, force_av."""
        v = (C.c_uint64 * 8)()
        self._check(self._lib.sph_pair_stats(self._h, v, 1 if reset else 0))
        return dict(density=v[0], wall=v[1], force_fluid=v[2], force_wall=v[3], force_av=v[4])


class Batch:
    """Many independent systems stepped together: each pair of steps is one
    CUDA-graph launch whose branches (one per member) overlap on the device.
    Members keep their own state; results equal stepping each alone."""

    def __init__(self, members):
        self._lib = L.load()
        self.members = list(members)
        arr = (C.c_void_p * len(self.members))(*[m._h.value for m in self.members])
        h = C.c_void_p()
        rc = self._lib.sph_batch_create(arr, len(self.members), C.byref(h))
        if rc != 0:
            raise SphError(rc, "sph_batch_create failed (members must hold particles, one device)")
        self._h = h
        self.fused = (len({m.precision for m in self.members}) == 1 and
                      self.members[0].precision == MIXED and
                      len({m.dim for m in self.members}) == 1)

    def _check(self, rc):
        if rc != 0:
            msg = self._lib.sph_batch_last_error(self._h)
            raise SphError(rc, msg.decode() if msg else "")

    def step(self, nsteps: int = 2):
        self._check(self._lib.sph_batch_step(self._h, int(nsteps)))

    def set_tuning(self, warps_per_block: int):
        """Warps per block of the fused pair passes (2, 4 or 8)."""
        self._check(self._lib.sph_batch_set_tuning(self._h, int(warps_per_block)))

    def set_fused(self, on: bool):
        """Fused steps (one launch per kernel over all members; the default
        for mixed-precision members of one dimension) or one graph branch per
        member.  Results are the same."""
        self._check(self._lib.sph_batch_set_fused(self._h, 1 if on else 0))
        self.fused = bool(on)

    def synchronize(self):
        self._check(self._lib.sph_batch_synchronize(self._h))

    def stream(self) -> int:
        p = C.c_void_p()
        self._check(self._lib.sph_batch_stream(self._h, C.byref(p)))
        return p.value or 0

    def idle(self) -> bool:
        """True when everything the batch and its members queued has
        finished (never waits)."""
        i = C.c_int()
        self._check(self._lib.sph_batch_query(self._h, C.byref(i)))
        return bool(i.value)

    def stats(self) -> dict:
        a, b_, c = C.c_int64(), C.c_int64(), C.c_int64()
        self._check(self._lib.sph_batch_stats(self._h, C.byref(a), C.byref(b_), C.byref(c)))
        return dict(kernels_per_graph=a.value, graph_launches=b_.value, kernels=c.value)

    def close(self):
        if getattr(self, "_h", None):
            self._lib.sph_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


MAT_KERNEL = L.SPH_MAT_KERNEL
MAT_PROJECTION = L.SPH_MAT_PROJECTION
VEC_PROJECTION = L.SPH_VEC_PROJECTION


class CsrMatrix:
    """A device-resident sparse matrix from ``assemble_matrix`` (CSR, rows
    and columns in reference particle order, columns ascending per row)."""

    def __init__(self, handle):
        self._lib = L.load()
        self._h = handle
        n, nnz = C.c_int64(), C.c_int64()
        self._lib.sph_csr_info(self._h, C.byref(n), C.byref(nnz))
        self.n, self.nnz = n.value, nnz.value

    def arrays(self):
        """(row_ptr int64[n+1], col int32[nnz], val float64[nnz]) on the host."""
        rp = np.empty(self.n + 1, np.int64)
        col = np.empty(self.nnz, np.int32)
        val = np.empty(self.nnz, np.float64)
        rc = self._lib.sph_csr_download(self._h, _ptr(rp), _ptr(col), _ptr(val))
        if rc != 0:
            raise SphError(rc, "sph_csr_download failed")
        return rp, col, val

    def to_scipy(self):
        import scipy.sparse as sp
        rp, col, val = self.arrays()
        return sp.csr_matrix((val, col, rp), shape=(self.n, self.n))

    def cg(self, b, reltol: float = float(np.sqrt(np.finfo(np.float64).eps)), maxiter: int = -1):
        """cg(A, b) of IterativeSolvers (x0 = 0, ||r|| <= reltol ||b||) on the
        device; returns (x, iterations, final residual norm)."""
        b = np.ascontiguousarray(b, dtype=np.float64).reshape(self.n)
        x = np.empty(self.n, np.float64)
        it, res = C.c_int32(), C.c_double()
        rc = self._lib.sph_cg(self._h, _ptr(b), _ptr(x), float(reltol), int(maxiter),
                              C.byref(it), C.byref(res))
        if rc != 0:
            raise SphError(rc, "sph_cg failed")
        return x, it.value, res.value

    def close(self):
        if getattr(self, "_h", None):
            self._lib.sph_csr_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def assemble_matrix(system: "ParticleSystem", func: int, param: float = 0.0) -> CsrMatrix:
    """assemble_matrix(sys, func) (core.jl:196-225) with a built-in function:
    MAT_KERNEL (W) or MAT_PROJECTION (the ISPH projection matrix; param =
    C_free).  Needs a current cell list."""
    h = C.c_void_p()
    system._check(system._lib.sph_assemble_matrix(system._h, int(func), float(param), C.byref(h)))
    return CsrMatrix(h)


def assemble_vector(system: "ParticleSystem", func: int) -> np.ndarray:
    """assemble_vector(sys, func) (core.jl:175-183) with a built-in function
    (VEC_PROJECTION), in reference particle order."""
    out = np.empty(system.n, np.float64)
    system._check(system._lib.sph_assemble_vector(system._h, int(func), _ptr(out)))
    return out


def shape_count(dim: int, shapes, device: int = 0) -> int:
    """Particles the device generator makes from ``shapes`` (no system needed)."""
    lib = L.load()
    arr = L.make_shapes(shapes)
    n = C.c_int64()
    rc = lib.sph_shape_count(int(device), int(dim), arr, len(shapes), C.byref(n))
    if rc != 0:
        raise SphError(rc, "sph_shape_count failed (invalid shape or no CUDA device)")
    return n.value


def generate_scratch(dim: int, shapes) -> int:
    """Temporary device bytes the device generator allocates for ``shapes``
    while it runs (host-side arithmetic)."""
    lib = L.load()
    arr = L.make_shapes(shapes)
    b = C.c_uint64()
    rc = lib.sph_generate_scratch(int(dim), arr, len(shapes), C.byref(b))
    if rc != 0:
        raise SphError(rc, "sph_generate_scratch: invalid shape")
    return b.value


def device_memory(device: int = 0) -> tuple:
    """(free, total) device bytes (cudaMemGetInfo)."""
    lib = L.load()
    f, t = C.c_uint64(), C.c_uint64()
    rc = lib.sph_device_memory(int(device), C.byref(f), C.byref(t))
    if rc != 0:
        raise SphError(rc, "sph_device_memory failed (no CUDA device)")
    return f.value, t.value


def memory_estimate(params: dict, n: int, precision: int = FP64) -> int:
    """Device bytes a system with these parameters holds with n particles
    (host-side arithmetic, no GPU needed).  Mixed precision: the exact
    allocation.  FP64: the rows are sized at the first density pass from
    the counts; the estimate gives them a full lattice neighbourhood per
    particle, an upper bound for a dam break (a clustering flow can need
    more)."""
    lib = L.load()
    p = L.make_params(L.sph_params, params, precision)
    b = C.c_uint64()
    rc = lib.sph_memory_estimate(C.byref(p), int(n), C.byref(b))
    if rc != 0:
        raise SphError(rc, "sph_memory_estimate: invalid parameters")
    return b.value


def arith_check(op: str, a, b=None, k: int = 59, device: int = 0):
    """The FP64 arithmetic the pair passes form on the integer pipes, applied
    on the device: op 'sub' (a - b through fixed-point copies at scale 2^k),
    'sqrt', 'rcp' (1/a) or 'two_over' (2/a).  For tests against IEEE results."""
    lib = L.load()
    code = {"sub": 0, "sqrt": 1, "rcp": 2, "two_over": 3}[op]
    a = np.ascontiguousarray(a, dtype=np.float64)
    bb = np.ascontiguousarray(b if b is not None else a, dtype=np.float64)
    if bb.shape != a.shape:
        raise ValueError("a and b must have the same shape")
    out = np.empty_like(a)
    rc = lib.sph_arith_check(device, code, int(k), int(a.size), a.ctypes.data, bb.ctypes.data,
                             out.ctypes.data)
    if rc != 0:
        raise SphError(rc, "sph_arith_check failed")
    return out


def pipe_peak(which: str, device: int = 0) -> float:
    """Measured issue rate (thread-instructions/s) of 'dfma', 'ffma', 'dadd',
    'i2f64' (int64 -> double conversion) or 'dfma_i2f' (FP64 FMAs, each with
    a conversion beside it: the FMA rate)."""
    lib = L.load()
    out = C.c_double()
    rc = lib.sph_pipe_peak(device, {"dfma": 0, "ffma": 1, "dadd": 2, "i2f64": 3, "dfma_i2f": 4}[which], C.byref(out))
    if rc != 0:
        raise SphError(rc, "sph_pipe_peak failed")
    return out.value


class ParticleField:
    """ParticleField(sys, :var) (structs.jl:118-125) as a whole-array view."""

    def __init__(self, sys: ParticleSystem, var: str):
        self.sys = sys
        self.var = var

    def __array__(self, dtype=None, copy=None):
        a = self.sys.get(self.var)
        return a if dtype is None else a.astype(dtype)

    def __len__(self):
        return self.sys.n

    def __getitem__(self, i):
        return self.sys.get(self.var)[i]


def create_cell_list(sys: ParticleSystem):
    """create_cell_list!(sys) -- core.jl:51-90."""
    sys.create_cell_list()


def apply(sys: ParticleSystem, op: Operator, self: bool = False):
    """apply!(sys, op!; self) -- core.jl:151-161: binary or unary by operator."""
    if op.binary:
        sys.apply(op, self)
    else:
        sys.apply_unary(op)


def apply_binary(sys: ParticleSystem, op: Operator):
    """apply_binary!(sys, op!) -- core.jl:125-129."""
    if not op.binary:
        raise SphError(L.SPH_ERR_ARG, f"{op.name} is not a pair operator")
    sys.apply(op, False)


def apply_unary(sys: ParticleSystem, op: Operator):
    """apply_unary!(sys, op!) -- core.jl:138-142."""
    if op.binary:
        raise SphError(L.SPH_ERR_ARG, f"{op.name} is not a unary operator")
    sys.apply_unary(op)


def sum(sys: ParticleSystem, func: SumFunction, x=None, particles=None):
    """sum(sys, func, x) (core.jl:240-260) at points, or sum(sys, func, p)
    (core.jl:271-291) for particles given by reference index."""
    if particles is not None:
        return sys.sum_particles(func, particles)
    return sys.sum_points(func, x)
