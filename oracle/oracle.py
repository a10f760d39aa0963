"""ctypes wrapper of the CPU oracle (liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, by the smoke check of
__graft_entry__ and by the CPU-baseline leg of bench.py, as the checker or the
timed CPU arm.  The GPU library never uses it.  See sph_oracle.h for what it
restates and how it is pinned.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")

ORC_FLUID, ORC_WALL = 0, 1
OP_DENSITY, OP_DENSITY_REF, OP_FORCE, OP_WALL_PRESSURE = 1, 2, 3, 4
OP_RESET_RHO, OP_RESET_RHO_REF, OP_RESET_A, OP_EOS, OP_KICK, OP_DRIFT, OP_HYDROSTATIC = range(10, 17)
SUM_DENSITY, SUM_KERNEL, SUM_PRESSURE, SUM_SHEPARD = 1, 2, 3, 4
MAT_KERNEL, MAT_PROJECTION = 1, 2
VEC_PROJECTION = 1


class orc_params(C.Structure):
    _fields_ = [
        ("dim", C.c_int32), ("precision", C.c_int32), ("h", C.c_double),
        ("domain_min", C.c_double * 3), ("domain_max", C.c_double * 3),
        ("mass", C.c_double), ("rho0", C.c_double), ("c0", C.c_double),
        ("h_smooth", C.c_double), ("alpha", C.c_double), ("eps_xsph", C.c_double),
        ("gravity", C.c_double * 3), ("dt", C.c_double), ("col_height", C.c_double),
        ("vertical_axis", C.c_int32),
        ("eos", C.c_int32),
    ]


def build(force: bool = False) -> str:
    if force or not os.path.exists(LIB_PATH) or \
            os.path.getmtime(LIB_PATH) < max(os.path.getmtime(os.path.join(HERE, f))
                                             for f in ("sph_oracle.c", "sph_oracle.h")):
        r = subprocess.run(["make", "-C", HERE, "-B" if force else "liboracle.so"],
                           capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    return LIB_PATH


_lib = None


def load():
    global _lib
    if _lib is not None:
        return _lib
    build()
    lib = C.CDLL(LIB_PATH)
    P, I64, DP = C.c_void_p, C.c_int64, C.c_void_p
    sig = {
        "orc_create": (P, [C.POINTER(orc_params)]),
        "orc_destroy": (None, [P]),
        "orc_dim": (C.c_int, [P]),
        "orc_geometry": (None, [P, C.POINTER(I64), C.POINTER(I64), C.POINTER(I64),
                                C.POINTER(I64), C.POINTER(C.c_int32)]),
        "orc_add_particles": (C.c_int, [P, I64, DP, DP, DP, DP, DP]),
        "orc_num_particles": (I64, [P]),
        "orc_get_state": (None, [P, DP, DP, DP, DP, DP, DP, DP, DP, DP]),
        "orc_set_state": (None, [P, DP, DP, DP, DP, DP, DP, DP]),
        "orc_find_key": (I64, [P, C.POINTER(C.c_double)]),
        "orc_create_cell_list": (None, [P]),
        "orc_apply": (I64, [P, C.c_int, C.c_int]),
        "orc_apply_unary": (None, [P, C.c_int]),
        "orc_sum_point": (None, [P, C.c_int, I64, DP, DP]),
        "orc_sum_particle": (None, [P, C.c_int, I64, DP, DP]),
        "orc_keys": (None, [P, DP]),
        "orc_pairs": (I64, [P, DP, I64]),
        "orc_assemble_matrix": (I64, [P, C.c_int, C.c_double, DP, DP, DP, I64]),
        "orc_assemble_vector": (None, [P, C.c_int, DP]),
        "orc_init": (I64, [P]),
        "orc_step": (I64, [P, C.c_int]),
        "orc_pair_passes_sample": (I64, [P, I64, I64]),
        "orc_num_threads": (C.c_int, []),
        "orc_kernel_w": (C.c_double, [C.c_int, C.c_double, C.c_double]),
        "orc_kernel_rdw": (C.c_double, [C.c_int, C.c_double, C.c_double]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def _p(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


def kernel_w(dim: int, h: float, r: float) -> float:
    return load().orc_kernel_w(dim, h, r)


def kernel_rdw(dim: int, h: float, r: float) -> float:
    return load().orc_kernel_rdw(dim, h, r)


def num_threads() -> int:
    return load().orc_num_threads()


class OracleSystem:
    """The reference's ParticleSystem restated on the CPU (reference order)."""

    def __init__(self, params: dict):
        self._lib = load()
        p = orc_params()
        p.dim = int(params["dim"])
        p.precision = 0
        p.h = float(params["h"])
        for d in range(3):
            p.domain_min[d] = float(params["domain_min"][d])
            p.domain_max[d] = float(params["domain_max"][d])
            p.gravity[d] = float(params["gravity"][d])
        for name in ("mass", "rho0", "c0", "h_smooth", "alpha", "eps_xsph", "dt", "col_height"):
            setattr(p, name, float(params[name]))
        p.vertical_axis = int(params["vertical_axis"])
        p.eos = int(params.get("eos", 0))
        self._h = self._lib.orc_create(C.byref(p))
        if not self._h:
            raise ValueError("invalid ParticleSystem declaration (h must be positive, "
                             "eos 0 or 1)")
        self.params = dict(params)

    def close(self):
        if getattr(self, "_h", None):
            self._lib.orc_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def geometry(self):
        kp = (C.c_int64 * 3)()
        kl = (C.c_int64 * 3)()
        km = C.c_int64()
        kd = (C.c_int64 * 27)()
        nd = C.c_int32()
        self._lib.orc_geometry(self._h, kp, kl, C.byref(km), kd, C.byref(nd))
        return dict(key_phase=tuple(kp), key_lim=tuple(kl), key_max=km.value,
                    key_diff=list(kd)[: nd.value])

    def add_particles(self, x, v=None, rho=None, rho_ref=None, type=None):
        x = np.ascontiguousarray(x, np.float64).reshape(-1, 3)
        n = x.shape[0]
        v = None if v is None else np.ascontiguousarray(v, np.float64).reshape(n, 3)
        rho = None if rho is None else np.ascontiguousarray(rho, np.float64)
        rr = None if rho_ref is None else np.ascontiguousarray(rho_ref, np.float64)
        t = None if type is None else np.ascontiguousarray(type, np.int32)
        self._lib.orc_add_particles(self._h, n, _p(x), _p(v), _p(rho), _p(rr), _p(t))

    @property
    def n(self) -> int:
        return self._lib.orc_num_particles(self._h)

    def state(self) -> dict:
        n = self.n
        out = dict(x=np.empty((n, 3)), v=np.empty((n, 3)), a=np.empty((n, 3)),
                   xsph=np.empty((n, 3)), rho=np.empty(n), rho_ref=np.empty(n), P=np.empty(n),
                   type=np.empty(n, np.int32), oid=np.empty(n, np.int64))
        self._lib.orc_get_state(self._h, *[_p(out[k]) for k in
                                          ("x", "v", "a", "xsph", "rho", "rho_ref", "P", "type", "oid")])
        return out

    def set_state(self, x=None, v=None, a=None, xsph=None, rho=None, rho_ref=None, P=None):
        conv = lambda q: None if q is None else np.ascontiguousarray(q, np.float64)
        arrs = [conv(q) for q in (x, v, a, xsph, rho, rho_ref, P)]
        self._lib.orc_set_state(self._h, *[_p(q) for q in arrs])

    def find_key(self, x) -> int:
        arr = (C.c_double * 3)(*[float(t) for t in x])
        return self._lib.orc_find_key(self._h, arr)

    def create_cell_list(self):
        self._lib.orc_create_cell_list(self._h)

    def apply(self, op: int, self_term: bool = False) -> int:
        r = self._lib.orc_apply(self._h, op, 1 if self_term else 0)
        if r < 0:
            raise RuntimeError("cell list is stale; call create_cell_list first")
        return r

    def apply_unary(self, op: int):
        self._lib.orc_apply_unary(self._h, op)

    def sum_points(self, func: int, x) -> np.ndarray:
        x = np.ascontiguousarray(x, np.float64).reshape(-1, 3)
        out = np.empty(x.shape[0])
        self._lib.orc_sum_point(self._h, func, x.shape[0], _p(x), _p(out))
        return out

    def assemble_matrix(self, func: int, param: float = 0.0):
        """(I, J, V) of assemble_matrix in the reference's push order."""
        n = self._lib.orc_assemble_matrix(self._h, func, float(param), None, None, None, 0)
        I = np.empty(n, np.int64)
        J = np.empty(n, np.int64)
        V = np.empty(n, np.float64)
        self._lib.orc_assemble_matrix(self._h, func, float(param), _p(I), _p(J), _p(V), n)
        return I, J, V

    def assemble_vector(self, func: int) -> np.ndarray:
        out = np.empty(self.n, np.float64)
        self._lib.orc_assemble_vector(self._h, func, _p(out))
        return out

    def sum_particles(self, func: int, idx) -> np.ndarray:
        idx = np.ascontiguousarray(idx, np.int64).reshape(-1)
        out = np.empty(idx.shape[0])
        self._lib.orc_sum_particle(self._h, func, idx.shape[0], _p(idx), _p(out))
        return out

    def keys(self) -> np.ndarray:
        out = np.empty(self.n, np.int64)
        self._lib.orc_keys(self._h, _p(out))
        return out

    def pairs(self) -> np.ndarray:
        cnt = self._lib.orc_pairs(self._h, None, 0)
        out = np.empty((cnt, 2), np.int64)
        if cnt:
            self._lib.orc_pairs(self._h, _p(out), cnt)
        return out

    def init_state(self) -> int:
        return self._lib.orc_init(self._h)

    def step(self, nsteps: int = 1) -> int:
        return self._lib.orc_step(self._h, int(nsteps))

    def pair_passes_sample(self, lo: int, hi: int) -> int:
        return self._lib.orc_pair_passes_sample(self._h, int(lo), int(hi))


def from_case(case) -> OracleSystem:
    s = OracleSystem(case.params)
    s.add_particles(case.x, case.v, type=case.type)
    return s
