"""sph_cell_list_noalloc: the cell-list build for callers that cannot let the
library allocate device memory (their GPU memory belongs to their own pool or
budget, e.g. CUDA.jl's allocator or a serving process admitting work against a
fixed HBM budget).  The entry point's scratch is one static device array shared
by every call, so the test checks it against the regular create_cell_list!
entry point on several calls in a row with different inputs: whatever the
previous call left in the scratch must not leak into the next result.

Integer outputs, so the comparison is exact.  This file is collected last on
purpose; it passes alone in a fresh process and after the other tests.
"""
import ctypes as C

import numpy as np
import pytest

import sphgpu
from sphgpu import _lib as L
from sphgpu import geometry as G

pytestmark = pytest.mark.gpu


def expected_from_regular_entry_point(case):
    """Cells as create_cell_list! builds them, read back through the regular
    C-ABI path: each particle's key (SPH_FIELD_KEY) and which particles
    survived (SPH_FIELD_OID)."""
    g = sphgpu.ParticleSystem(case.params)
    g.upload(case.x, case.v, type=case.type)
    g.create_cell_list()
    keys, oid = g.get("key"), g.get("oid")
    key_max = g.geometry()["key_max"]
    g.close()
    key_of = np.zeros(case.n, np.int64)
    key_of[oid] = keys
    inside = np.nonzero(key_of > 0)[0]
    outside = np.nonzero(key_of == 0)[0]
    order = inside[np.lexsort((-inside, key_of[inside]))]  # key up, index down
    counts = np.bincount(key_of[inside], minlength=key_max + 2)[: key_max + 2]
    cell_start = np.concatenate([[0], np.cumsum(counts)])[: key_max + 2]
    return key_max, cell_start, np.concatenate([order, outside[::-1]])


def run_noalloc(case, key_max):
    import torch
    lib = L.load()
    p = L.make_params(L.sph_params, case.params)
    dx = torch.from_numpy(np.ascontiguousarray(case.x, dtype=np.float64)).cuda()
    d_start = torch.full((key_max + 2,), -7, dtype=torch.int32, device="cuda")
    d_order = torch.full((case.n,), -7, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    rc = lib.sph_cell_list_noalloc(C.byref(p), case.n, C.c_void_p(dx.data_ptr()),
                                   C.c_void_p(d_start.data_ptr()), C.c_void_p(d_order.data_ptr()),
                                   None)
    torch.cuda.synchronize()
    assert rc == L.SPH_OK
    return d_start.cpu().numpy(), d_order.cpu().numpy()


def with_escapees(case, seed):
    rng = np.random.default_rng(seed)
    x = case.x.copy()
    idx = rng.choice(case.n, 25, replace=False)
    x[idx[:10], 0] = np.nan
    x[idx[10:], 1] = 1e3
    case.x = x
    return case


def test_noalloc_matches_regular_entry_point_on_consecutive_calls(gpu):
    cases = [with_escapees(G.dam_break(2, 0.02), 1),
             with_escapees(G.dam_break(3, 0.05), 2),
             G.dam_break(2, 0.02),
             G.dam_break(2, 0.04)]
    for case in cases:
        key_max, cs_ref, order_ref = expected_from_regular_entry_point(case)
        cs, order = run_noalloc(case, key_max)
        assert np.array_equal(cs, cs_ref)
        assert np.array_equal(order, order_ref)


def test_noalloc_rejects_sizes_beyond_its_scratch(gpu):
    lib = L.load()
    case = G.dam_break(2, 0.1)
    p = L.make_params(L.sph_params, case.params)
    dummy = C.c_void_p(16)  # never dereferenced: the size check comes first
    rc = lib.sph_cell_list_noalloc(C.byref(p), (1 << 20) + 1, dummy, dummy, dummy, None)
    assert rc == L.SPH_ERR_BUDGET
    p.h = 1e-4  # a 4 x 3 domain at h = 1e-4 needs 1.2e9 cells
    rc = lib.sph_cell_list_noalloc(C.byref(p), 10, dummy, dummy, dummy, None)
    assert rc == L.SPH_ERR_BUDGET
