"""Device-side particle generation (sph_generate) against the host restatement
of the reference's lattice rules: same particles, same order, bit for bit."""
import numpy as np
import pytest

import sphgpu
from sphgpu import geometry as G

pytestmark = pytest.mark.gpu

CASES = [
    (2, 0.02, {}),
    (2, 0.0071, dict(col_height=1.3)),
    (2, 0.013, dict(lid=True, col_width=0.7)),
    (3, 0.05, {}),
    (3, 0.03, dict(lid=True, depth=0.6)),
    (3, 0.041, dict(col_height=1.1, wall_layers=2)),
]


@pytest.mark.parametrize("dim,dr,kw", CASES)
def test_generate_matches_host(gpu, dim, dr, kw):
    host = G.dam_break(dim, dr, **kw)
    dev = G.dam_break_shapes(dim, dr, **kw)
    assert dev.params == host.params
    assert sphgpu.shape_count(dim, dev.shapes) == host.n
    g = sphgpu.ParticleSystem(dev.params, sphgpu.FP64)
    assert g.generate(dev.shapes) == host.n
    assert np.array_equal(g.get("x"), host.x)
    assert np.array_equal(g.get("type"), host.type)
    assert np.array_equal(g.get("v"), np.zeros_like(host.x))
    assert np.array_equal(g.get("oid"), np.arange(host.n))
    g.close()


def test_generated_system_steps_like_uploaded(gpu):
    host = G.dam_break(2, 0.03)
    dev = G.dam_break_shapes(2, 0.03)
    a = sphgpu.ParticleSystem(host.params, sphgpu.MIXED)
    a.upload(host.x, host.v, type=host.type)
    b = sphgpu.ParticleSystem(dev.params, sphgpu.MIXED)
    b.generate(dev.shapes)
    for s in (a, b):
        s.init_state()
        s.step(6)
    for f in ("x", "v", "rho", "P", "a"):
        assert np.array_equal(a.get(f), b.get(f)), f


def test_bad_shapes_raise(gpu):
    dev = G.dam_break_shapes(2, 0.05)
    g = sphgpu.ParticleSystem(dev.params, sphgpu.FP64)
    bad = [dict(dev.shapes[0], dr=-1.0)]
    with pytest.raises(sphgpu.SphError):
        g.generate(bad)
    bad3 = [dict(dev.shapes[0], lo=(0.0, 0.0, 0.5), hi=(1.0, 1.0, 0.5))]  # z != 0 in 2D
    with pytest.raises(sphgpu.SphError):
        g.generate(bad3)
