"""Fields through pinned host buffers (the ``out=`` path of the e2e loop)
give the same bits as through freshly allocated pageable arrays: every
field read after steps with removals, and every settable field written
before further steps."""
import numpy as np
import pytest

import sphgpu
from sphgpu import geometry as G

pytestmark = pytest.mark.gpu

FIELDS_GET = ("x", "v", "a", "xsph", "rho", "rho_ref", "P", "type", "oid", "key")
FIELDS_SET = ("x", "v", "a", "xsph", "rho", "rho_ref", "P", "type")


def pinned_like(a):
    torch = pytest.importorskip("torch")
    t = torch.empty(a.shape, dtype=getattr(torch, str(a.dtype)), pin_memory=True)
    return t.numpy()


@pytest.mark.parametrize("dim,dr,prec", [(2, 0.02, "fp64"), (3, 0.05, "fp64"), (3, 0.05, "mixed")])
def test_pinned_fields_equal_pageable(gpu, dim, dr, prec):
    c = G.dam_break(dim, dr)
    p = sphgpu.FP64 if prec == "fp64" else sphgpu.MIXED
    g = sphgpu.ParticleSystem(c.params, p)
    x = c.x.copy()
    x[7, 0] = np.nan          # removed by the next binning (tail fill)
    g.upload(x, c.v, type=c.type)
    g.init_state()
    g.step(3)
    for f in FIELDS_GET:
        ref = g.get(f)
        out = pinned_like(ref)
        out[...] = 0
        got = g.get(f, out=out)
        assert got is out
        assert np.array_equal(ref.view(np.uint8), out.view(np.uint8)), f

    # the same writes through both kinds of buffer, then more steps
    h = sphgpu.ParticleSystem(c.params, p)
    h.upload(x, c.v, type=c.type)
    h.init_state()
    h.step(3)
    rng = np.random.default_rng(3)
    for f in FIELDS_SET:
        base = g.get(f)
        if f == "type":
            vals = base
        elif f == "x":
            vals = base + rng.uniform(-1e-4, 1e-4, base.shape) * (np.arange(3) < dim)
        else:
            vals = base * (1.0 + rng.uniform(-1e-3, 1e-3, base.shape))
        g.set(f, vals)                   # pageable
        pin = pinned_like(np.ascontiguousarray(vals))
        pin[...] = vals
        h.set(f, pin)                    # pinned
    g.step(2)
    h.step(2)
    for f in FIELDS_GET:
        assert np.array_equal(g.get(f).view(np.uint8), h.get(f).view(np.uint8)), f
    g.close()
    h.close()


@pytest.mark.parametrize("prec,pin", [("fp64", True), ("fp64", False), ("mixed", True)])
def test_step_io_equals_set_step_get(gpu, prec, pin):
    """sph_step_io: the inputs set, one step, the outputs read (some of them
    while the step still runs) give the bits of set_field + step + get_field,
    also in a step that removes a particle leaving the box."""
    c = G.dam_break(3, 0.05)
    p = sphgpu.FP64 if prec == "fp64" else sphgpu.MIXED
    sysA = sphgpu.ParticleSystem(c.params, p)
    sysB = sphgpu.ParticleSystem(c.params, p)
    for s in (sysA, sysB):
        s.upload(c.x, c.v, type=c.type)
        s.init_state()
        s.step(2)
    outs_names = ("x", "rho", "P", "v", "a", "xsph", "type", "oid", "rho_ref", "key")
    for k in range(3):
        inp = {f: sysA.get(f) for f in ("x", "v", "a", "xsph")}
        if k == 1:
            # a fluid particle sent far outside the box: removed by this step's binning
            i = int(np.nonzero(sysA.get("type") == 0)[0][5])
            inp["x"][i] = [50.0, 50.0, 50.0]
        for f, a in inp.items():
            sysA.set(f, a)
        sysA.step(1)
        want = {f: sysA.get(f) for f in outs_names}
        n0 = sysB.n
        outs = {}
        for f in outs_names:
            ref = sysB.get(f)
            outs[f] = pinned_like(ref) if pin else np.empty_like(ref)
        sysB.step_io(inp, outs)
        n1 = sysB.n
        assert n1 == sysA.n and n1 <= n0
        for f in outs_names:
            assert np.array_equal(outs[f][:n1].view(np.uint8), want[f].view(np.uint8)), (k, f)
    sysA.close()
    sysB.close()
