"""Mixed-precision path against the FP64 path on identical inputs.

The mixed path classifies candidates exactly like the FP64 path, so its pair
set (and pair counts per category) must be identical for the same positions.
Its arithmetic is FP32 with FP64 accumulation per batch of <= 16 hits, so the
fields differ from FP64 by the FP32 rounding of each term; the tolerances
below are the stated per-field accuracy of the mixed path, about 5x the
errors measured on GB300 (after the initialisation: rho 2.0e-7, P 3.0e-7,
a 5.3e-7; after 10 steps: x 2.0e-7 dr):
  rho (density sum)          max relative error      <= 1e-6
  P (Tait, fluid)            max |dP| / max|P|        <= 2e-6
  a (acceleration)           ||da|| / ||a||           <= 5e-6
  xsph (one step, same state) ||dxsph|| / ||xsph||    <= 1e-5
  x after 10 steps           max |dx| / dr            <= 1e-6
"""
import numpy as np
import pytest

import sphgpu
from sphgpu import geometry as G

pytestmark = pytest.mark.gpu


def pair_of_systems(case):
    out = []
    for prec in (sphgpu.FP64, sphgpu.MIXED):
        g = sphgpu.ParticleSystem(case.params, prec)
        g.upload(case.x, case.v, type=case.type)
        out.append(g)
    return out


def errors(a, b):
    d = {}
    for f in ("rho", "P", "a", "xsph"):
        x, y = a.get(f), b.get(f)
        if x.ndim == 2:
            d[f] = np.linalg.norm(x - y) / max(np.linalg.norm(x), 1e-300)
        elif f == "P":
            d[f] = np.abs(x - y).max() / max(np.abs(x).max(), 1e-300)
        else:
            fl = a.get("type") == 0
            d[f] = (np.abs(x - y)[fl] / np.abs(x)[fl]).max()
    return d


@pytest.mark.parametrize("dim,dr", [(2, 0.02), (3, 0.04)])
def test_mixed_init_accuracy_and_pairs(gpu, dim, dr):
    c = G.dam_break(dim, dr)
    g64, g32 = pair_of_systems(c)
    g64.init_state()
    g32.init_state()
    assert g64.pair_count() == g32.pair_count()
    assert g64.pair_stats() == g32.pair_stats()
    e = errors(g64, g32)
    print(f"\nmixed vs fp64 after init ({dim}D dr={dr}): {e}")
    assert e["rho"] <= 1e-6
    assert e["P"] <= 2e-6
    assert e["a"] <= 5e-6


@pytest.mark.parametrize("dim,dr", [(2, 0.02), (3, 0.04)])
def test_mixed_steps(gpu, dim, dr):
    c = G.dam_break(dim, dr)
    g64, g32 = pair_of_systems(c)
    for g in (g64, g32):
        g.init_state()
        g.pair_count(reset=True)
        g.step(10)
    dx = np.abs(g64.get("x") - g32.get("x")).max()
    print(f"\nmixed vs fp64 after 10 steps ({dim}D dr={dr}): max|dx|/dr = {dx / dr:.3e}")
    assert dx / dr <= 1e-6
    assert g64.n == g32.n
    # one more step from the identical FP64 state (reference density
    # included): the per-step error of the mixed arithmetic.  The Tait EOS
    # turns a density error d into a pressure error 7 B d (~0.5 Pa here), so
    # P and a are bounded relative to their largest values.
    for f in ("x", "v", "a", "xsph", "rho_ref"):
        g32.set(f, g64.get(f))
    g64.step(1)
    g32.step(1)
    e = errors(g64, g32)
    print(f"mixed vs fp64, one step from the same state: {e}")
    assert e["rho"] <= 1e-6 and e["P"] <= 2e-4 and e["a"] <= 5e-4 and e["xsph"] <= 1e-5
    g32.synchronize()


def test_mixed_reference_style_operators(gpu):
    """apply!/apply_unary! in mixed precision: the FP32 neighbour copies are
    rebuilt when the state changed outside a fused density pass."""
    c = G.dam_break(2, 0.04)
    g64, g32 = pair_of_systems(c)
    for g in (g64, g32):
        g.create_cell_list()
        sphgpu.apply(g, sphgpu.reset_rho0)
        sphgpu.apply(g, sphgpu.find_rho0, self=True)
        sphgpu.apply(g, sphgpu.hydrostatic)
        sphgpu.apply(g, sphgpu.reset_rho)
        sphgpu.apply(g, sphgpu.find_rho, self=True)
        sphgpu.apply(g, sphgpu.find_pressure)
        sphgpu.apply(g, sphgpu.wall_pressure)
        sphgpu.apply(g, sphgpu.reset_a)
        sphgpu.apply(g, sphgpu.internal_force)
    e = errors(g64, g32)
    assert e["rho"] <= 1e-6 and e["a"] <= 5e-6
