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
