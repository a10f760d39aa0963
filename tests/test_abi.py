"""The C-ABI library loads, exports every entry point include/sphgpu.h
declares, lays out sph_params as the header does, and rejects invalid calls
before touching a GPU (these tests run without one)."""
import ctypes as C
import os
import re
import subprocess
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "sphgpu.h")


def declared_functions():
    src = open(HEADER).read()
    return sorted(set(re.findall(r"^(?:int|const char\*)\s+(sph_\w+)\(", src, re.M)))


def test_header_declares_entry_points():
    names = declared_functions()
    for required in ("sph_create", "sph_create_cell_list", "sph_apply", "sph_apply_unary",
                     "sph_sum_point", "sph_sum_particle", "sph_step", "sph_upload",
                     "sph_get_field", "sph_set_field", "sph_destroy"):
        assert required in names


def test_library_exports_every_declared_symbol(sph_lib):
    from sphgpu import _lib
    for name in declared_functions():
        assert hasattr(sph_lib, name), name
        assert name in _lib.PROTOTYPES, f"{name} has no ctypes prototype"


def test_params_layout_matches_header(sph_lib):
    from sphgpu import _lib
    prog = r'''
#include <stdio.h>
#include <stddef.h>
#include "sphgpu.h"
int main(void) {
  printf("%zu %zu %zu %zu %zu\n", sizeof(sph_params), offsetof(sph_params, h),
         offsetof(sph_params, gravity), offsetof(sph_params, col_height),
         offsetof(sph_params, vertical_axis));
  return 0;
}
'''
    with tempfile.TemporaryDirectory() as td:
        c = os.path.join(td, "p.c")
        exe = os.path.join(td, "p")
        open(c, "w").write(prog)
        subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), c, "-o", exe], check=True)
        got = [int(t) for t in subprocess.run([exe], capture_output=True, text=True).stdout.split()]
    P = _lib.sph_params
    assert got == [C.sizeof(P), P.h.offset, P.gravity.offset, P.col_height.offset,
                   P.vertical_axis.offset]


def test_invalid_calls_fail_without_gpu(sph_lib):
    from sphgpu import _lib
    assert sph_lib.sph_abi_version() == 2
    assert sph_lib.sph_destroy(None) == _lib.SPH_ERR_ARG
    assert sph_lib.sph_last_error(None) == b"null handle"
    p = _lib.sph_params()
    p.dim = 5
    p.h = 0.1
    h = C.c_void_p()
    assert sph_lib.sph_create(C.byref(p), 0, C.byref(h)) == _lib.SPH_ERR_ARG
    p.dim = 2
    p.h = -1.0  # structs.jl:59 asserts h > 0
    assert sph_lib.sph_create(C.byref(p), 0, C.byref(h)) == _lib.SPH_ERR_ARG
    assert sph_lib.sph_apply(None, 1, 0) == _lib.SPH_ERR_ARG
    assert sph_lib.sph_step(None, 1) == _lib.SPH_ERR_ARG


def test_missing_library_fails_loudly(tmp_path):
    from sphgpu import _lib
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        _lib.load(str(tmp_path / "absent.so"))
