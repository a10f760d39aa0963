"""ctypes binding of libsphgpu.so (the C ABI declared in include/sphgpu.h).

The library is built in-tree (``smoothedparticles.jl_gb300/libsphgpu.so``) by
``sphgpu.build.build_library``.  Loading fails loudly when it is missing: there
is no CPU fallback for any operation.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
PKG_ROOT = os.path.dirname(HERE)
LIB_PATH = os.path.join(PKG_ROOT, "libsphgpu.so")

# status codes
SPH_OK = 0
SPH_ERR_ARG = -1
SPH_ERR_CUDA = -2
SPH_ERR_STATE = -3
SPH_ERR_NOMEM = -4
SPH_ERR_DEVICE = -5
SPH_ERR_UNSUPPORTED = -6
SPH_ERR_TIMEOUT = -7
SPH_ERR_BUDGET = -8

SPH_FLUID = 0
SPH_WALL = 1
SPH_PREC_FP64 = 0
SPH_PREC_MIXED = 1

SPH_OP_DENSITY = 1
SPH_OP_DENSITY_REF = 2
SPH_OP_FORCE = 3
SPH_OP_WALL_PRESSURE = 4
SPH_OP_RESET_RHO = 10
SPH_OP_RESET_RHO_REF = 11
SPH_OP_RESET_A = 12
SPH_OP_EOS = 13
SPH_OP_KICK = 14
SPH_OP_DRIFT = 15
SPH_OP_HYDROSTATIC = 16

SPH_SUM_DENSITY = 1
SPH_SUM_KERNEL = 2
SPH_SUM_PRESSURE = 3
SPH_SUM_SHEPARD = 4

SPH_FIELD_X = 1
SPH_FIELD_V = 2
SPH_FIELD_A = 3
SPH_FIELD_XSPH = 4
SPH_FIELD_RHO = 5
SPH_FIELD_RHO_REF = 6
SPH_FIELD_P = 7
SPH_FIELD_TYPE = 8
SPH_FIELD_OID = 9
SPH_FIELD_KEY = 10

KERNEL_NAMES = ["bin_keys", "bin_remove", "bin_scan", "bin_scatter", "bin_rank", "bin_gather",
                "density", "force", "unary", "sum", "io", "wall_pressure"]
SPH_KERNEL_COUNT = len(KERNEL_NAMES)


class sph_params(C.Structure):
    _fields_ = [
        ("dim", C.c_int32),
        ("precision", C.c_int32),
        ("h", C.c_double),
        ("domain_min", C.c_double * 3),
        ("domain_max", C.c_double * 3),
        ("mass", C.c_double),
        ("rho0", C.c_double),
        ("c0", C.c_double),
        ("h_smooth", C.c_double),
        ("alpha", C.c_double),
        ("eps_xsph", C.c_double),
        ("gravity", C.c_double * 3),
        ("dt", C.c_double),
        ("col_height", C.c_double),
        ("vertical_axis", C.c_int32),
        ("eos", C.c_int32),
        ("cell_factor", C.c_double),
    ]


SPH_EOS_TAIT = 0
SPH_EOS_LINEAR = 1

SPH_MAT_KERNEL = 1
SPH_MAT_PROJECTION = 2
SPH_VEC_PROJECTION = 1

SPH_SHAPE_BOX = 1
SPH_SHAPE_LAYER = 2


class sph_shape(C.Structure):
    _fields_ = [
        ("kind", C.c_int32),
        ("type", C.c_int32),
        ("dr", C.c_double),
        ("lo", C.c_double * 3),
        ("hi", C.c_double * 3),
        ("width", C.c_double),
        ("keep_axis", C.c_int32),
        ("reserved", C.c_int32),
        ("keep_max", C.c_double),
    ]


def make_shapes(shapes) -> "C.Array":
    """An array of sph_shape from dicts (kind 'box' or 'layer')."""
    arr = (sph_shape * max(1, len(shapes)))()
    for i, d in enumerate(shapes):
        s = arr[i]
        s.kind = SPH_SHAPE_BOX if d["kind"] == "box" else SPH_SHAPE_LAYER
        s.type = int(d["type"])
        s.dr = float(d["dr"])
        for k in range(3):
            s.lo[k] = float(d["lo"][k])
            s.hi[k] = float(d["hi"][k])
        s.width = float(d.get("width", 0.0))
        s.keep_axis = int(d.get("keep_axis", -1))
        s.reserved = 0
        s.keep_max = float(d.get("keep_max", 0.0))
    return arr


def make_params(cls, p: dict, precision: int = 0):
    """Fills a params structure (``sph_params`` or the oracle's twin) from a dict."""
    s = cls()
    s.dim = int(p["dim"])
    s.precision = int(precision)
    s.h = float(p["h"])
    for d in range(3):
        s.domain_min[d] = float(p["domain_min"][d])
        s.domain_max[d] = float(p["domain_max"][d])
        s.gravity[d] = float(p["gravity"][d])
    for name in ("mass", "rho0", "c0", "h_smooth", "alpha", "eps_xsph", "dt", "col_height"):
        setattr(s, name, float(p[name]))
    s.vertical_axis = int(p["vertical_axis"])
    s.eos = int(p.get("eos", SPH_EOS_TAIT))
    if any(f[0] == "cell_factor" for f in cls._fields_):
        s.cell_factor = float(p.get("cell_factor", 0.0))
    return s


_P = C.c_void_p
_I64 = C.c_int64
_I32 = C.c_int32
_DP = C.POINTER(C.c_double)

# name -> (restype, argtypes)
PROTOTYPES = {
    "sph_abi_version": (C.c_int, []),
    "sph_last_error": (C.c_char_p, [_P]),
    "sph_create": (C.c_int, [C.POINTER(sph_params), C.c_int, C.POINTER(_P)]),
    "sph_destroy": (C.c_int, [_P]),
    "sph_geometry": (C.c_int, [_P, C.POINTER(_I64), C.POINTER(_I64), C.POINTER(_I64),
                               C.POINTER(_I64), C.POINTER(_I32)]),
    "sph_upload": (C.c_int, [_P, _I64, _P, _P, _P, _P, _P]),
    "sph_num_particles": (C.c_int, [_P, C.POINTER(_I64)]),
    "sph_get_field": (C.c_int, [_P, C.c_int, _P]),
    "sph_set_field": (C.c_int, [_P, C.c_int, _P]),
    "sph_create_cell_list": (C.c_int, [_P]),
    "sph_apply": (C.c_int, [_P, C.c_int, C.c_int]),
    "sph_apply_unary": (C.c_int, [_P, C.c_int]),
    "sph_sum_point": (C.c_int, [_P, C.c_int, _I64, _P, _P]),
    "sph_sum_particle": (C.c_int, [_P, C.c_int, _I64, _P, _P]),
    "sph_step": (C.c_int, [_P, C.c_int]),
    "sph_step_io": (C.c_int, [_P, C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p,
                              C.c_void_p]),
    "sph_init_state": (C.c_int, [_P]),
    "sph_pair_count": (C.c_int, [_P, C.POINTER(C.c_uint64), C.c_int]),
    "sph_synchronize": (C.c_int, [_P]),
    "sph_stream": (C.c_int, [_P, C.POINTER(_P)]),
    "sph_debug_pairs": (C.c_int, [_P, _P, _I64, C.POINTER(_I64)]),
    "sph_debug_hits": (C.c_int, [_P, _P, _I64, C.POINTER(_I64)]),
    "sph_set_profiling": (C.c_int, [_P, C.c_int]),
    "sph_kernel_stats": (C.c_int, [_P, C.c_int, C.POINTER(C.c_double), C.POINTER(_I64)]),
    "sph_reset_kernel_stats": (C.c_int, [_P]),
    "sph_launch_count": (C.c_int, [_P, C.POINTER(_I64)]),
    "sph_pair_stats": (C.c_int, [_P, C.POINTER(C.c_uint64), C.c_int]),
    "sph_pipe_peak": (C.c_int, [C.c_int, C.c_int, C.POINTER(C.c_double)]),
    "sph_arith_check": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                                  C.c_void_p]),
    "sph_cell_list_noalloc": (C.c_int, [C.POINTER(sph_params), _I64, _P, _P, _P, _P]),
    "sph_set_tuning": (C.c_int, [_P, C.c_int]),
    "sph_set_chunk_threads": (C.c_int, [_P, C.c_int]),
    "sph_get_chunk_threads": (C.c_int, [_P, C.POINTER(C.c_int)]),
    "sph_get_tuning": (C.c_int, [_P, C.POINTER(C.c_int)]),
    "sph_batch_create": (C.c_int, [C.POINTER(_P), C.c_int, C.POINTER(_P)]),
    "sph_batch_destroy": (C.c_int, [_P]),
    "sph_batch_last_error": (C.c_char_p, [_P]),
    "sph_batch_step": (C.c_int, [_P, C.c_int]),
    "sph_batch_synchronize": (C.c_int, [_P]),
    "sph_batch_stats": (C.c_int, [_P, C.POINTER(_I64), C.POINTER(_I64), C.POINTER(_I64)]),
    "sph_batch_stream": (C.c_int, [_P, C.POINTER(_P)]),
    "sph_batch_set_fused": (C.c_int, [_P, C.c_int]),
    "sph_batch_set_tuning": (C.c_int, [_P, C.c_int]),
    "sph_memory_estimate": (C.c_int, [C.POINTER(sph_params), _I64, C.POINTER(C.c_uint64)]),
    "sph_generate_scratch": (C.c_int, [C.c_int, _P, C.c_int, C.POINTER(C.c_uint64)]),
    "sph_device_memory": (C.c_int, [C.c_int, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]),
    "sph_batch_query": (C.c_int, [_P, C.POINTER(C.c_int)]),
    "sph_memory_usage": (C.c_int, [_P, C.POINTER(C.c_uint64)]),
    "sph_query": (C.c_int, [_P, C.POINTER(C.c_int)]),
    "sph_assemble_matrix": (C.c_int, [_P, C.c_int, C.c_double, C.POINTER(_P)]),
    "sph_assemble_vector": (C.c_int, [_P, C.c_int, _P]),
    "sph_csr_info": (C.c_int, [_P, C.POINTER(_I64), C.POINTER(_I64)]),
    "sph_csr_download": (C.c_int, [_P, _P, _P, _P]),
    "sph_csr_destroy": (C.c_int, [_P]),
    "sph_cg": (C.c_int, [_P, _P, _P, C.c_double, _I32, C.POINTER(_I32), C.POINTER(C.c_double)]),
    "sph_vtk_open": (C.c_int, [_P, C.c_char_p, C.POINTER(_P)]),
    "sph_vtk_save_frame": (C.c_int, [_P, C.c_uint, C.c_double, C.POINTER(_I32)]),
    "sph_vtk_frames": (C.c_int, [_P, C.POINTER(_I32)]),
    "sph_vtk_close": (C.c_int, [_P]),
    "sph_generate": (C.c_int, [_P, C.POINTER(sph_shape), C.c_int, C.POINTER(_I64)]),
    "sph_shape_count": (C.c_int, [C.c_int, C.c_int, C.POINTER(sph_shape), C.c_int,
                                  C.POINTER(_I64)]),
}

_lib = None


def load(path: str | None = None):
    """Loads libsphgpu.so (once) and declares every prototype."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or os.environ.get("SPHGPU_LIB", LIB_PATH)
    if not os.path.exists(p):
        raise RuntimeError(
            f"libsphgpu.so not found at {p}: build it first (sphgpu.build.build_library()); "
            "there is no CPU fallback")
    lib = C.CDLL(p)
    for name, (res, args) in PROTOTYPES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    if path is None:
        _lib = lib
    return lib
