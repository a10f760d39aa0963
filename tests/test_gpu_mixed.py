"""Mixed-precision path against the FP64 path on identical inputs.

The mixed path classifies candidates exactly like the FP64 path, so its pair
set (and pair counts per category) must be identical for the same positions.
Its arithmetic is FP32 with FP64 accumulation per batch of <= 32 hits, so the
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


def _oracle_state_after(oracle_mod, case, steps):
    o = oracle_mod.from_case(case)
    if steps:
        o.init_state()
        o.step(steps)
    o.create_cell_list()
    return o, o.state()


@pytest.mark.parametrize("dim,dr,steps", [(2, 0.02, 0), (3, 0.05, 0), (2, 0.02, 20), (3, 0.05, 4)])
def test_pair_set_of_both_paths_equals_oracle(gpu, oracle_mod, dim, dr, steps):
    """The set of neighbour pairs the density pass acts on and stores for the
    force pass -- the mixed path's hit masks and the FP64 path's rows, read
    back with sph_debug_hits -- equals the oracle's pair list (core.jl:94-112:
    every q with r <= h, q != p, in key_diff order) for every fluid target:
    the FP64 path's order included, the mixed path's as a set (its cell grid
    is offset from the reference's, so its neighbour order is its own).  Both
    on the initial lattice (many pairs exactly at r = h) and on the oracle's
    particles after some steps (off-lattice)."""
    c = G.dam_break(dim, dr)
    o, st = _oracle_state_after(oracle_mod, c, steps)
    ref = o.pairs()
    ref = ref[st["type"][ref[:, 0]] == G.FLUID]
    assert len(ref) > 0
    for prec in (sphgpu.MIXED, sphgpu.FP64):
        g = sphgpu.ParticleSystem(c.params, prec)
        g.upload(st["x"], st["v"], type=st["type"])
        g.create_cell_list()
        # an FP64 system's first density pass sizes its rows (it traverses,
        # having none): the second one stores its pairs in them
        for _ in range(2):
            sphgpu.apply(g, sphgpu.reset_rho)
            sphgpu.apply(g, sphgpu.find_rho, self=True)
        hits = g.debug_hits()
        assert hits.shape == ref.shape, (prec, hits.shape, ref.shape)
        if prec == sphgpu.MIXED:
            key = lambda a: a[np.lexsort((a[:, 1], a[:, 0]))]
            assert np.array_equal(key(hits), key(ref)), prec
        else:
            assert np.array_equal(hits, ref), prec
        g.close()


@pytest.mark.parametrize("dim,dr", [(2, 0.02), (3, 0.05)])
def test_mixed_error_against_oracle(gpu, oracle_mod, dim, dr):
    """The mixed path's per-field error measured against the oracle itself
    (the FP64 path equals the oracle bit for bit, so these are the errors of
    the mixed arithmetic), after the initial state and after 10 steps, with
    the bounds stated at the top of this file."""
    c = G.dam_break(dim, dr)
    g = sphgpu.ParticleSystem(c.params, sphgpu.MIXED)
    g.upload(c.x, c.v, type=c.type)
    o = oracle_mod.from_case(c)
    g.init_state()
    o.init_state()

    def err():
        st = o.state()
        fl = st["type"] == G.FLUID
        d = {}
        for f in ("rho", "P", "a"):
            x, y = st[f], g.get(f)
            if x.ndim == 2:
                d[f] = np.linalg.norm(x - y) / max(np.linalg.norm(x), 1e-300)
            elif f == "P":
                d[f] = np.abs(x - y).max() / max(np.abs(x).max(), 1e-300)
            else:
                d[f] = (np.abs(x - y)[fl] / np.abs(x)[fl]).max()
        d["x_over_dr"] = np.abs(st["x"] - g.get("x")).max() / dr
        return d
    e0 = err()
    print(f"\nmixed vs oracle after init ({dim}D dr={dr}): {e0}")
    assert e0["rho"] <= 1e-6 and e0["P"] <= 2e-6 and e0["a"] <= 5e-6 and e0["x_over_dr"] == 0.0
    g.step(10)
    o.step(10)
    e1 = err()
    print(f"mixed vs oracle after 10 steps: {e1}")
    assert g.n == o.n
    assert e1["x_over_dr"] <= 1e-6
    g.close()


@pytest.mark.parametrize("dim,dr,steps,factor", [(2, 0.02, 0, 1.25), (2, 0.02, 20, 1.6),
                                                 (2, 0.02, 20, 2.0), (3, 0.05, 0, 1.25),
                                                 (3, 0.05, 4, 1.2), (3, 0.05, 4, 2.0)])
def test_larger_cells_keep_the_pair_set(gpu, oracle_mod, dim, dr, steps, factor):
    """A mixed system with cells of factor * h (sph_params.cell_factor): the
    pair set the density pass acts on is still the oracle's (as a set: the
    neighbour order follows the larger cells), and the fields stay within
    the mixed path's bounds of the oracle after the initial state.  In 3D a
    factor of 2 puts ~512 particles in a cell, more chunks per work item
    than the stored hit masks take: those targets traverse in the force pass
    too (same results), and sph_debug_hits, which lists stored masks only,
    refuses -- the fields are checked there."""
    c = G.dam_break(dim, dr)
    o, st = _oracle_state_after(oracle_mod, c, steps)
    ref = o.pairs()
    ref = ref[st["type"][ref[:, 0]] == G.FLUID]
    params = dict(c.params, cell_factor=factor)
    g = sphgpu.ParticleSystem(params, sphgpu.MIXED)
    g.upload(st["x"], st["v"], type=st["type"])
    g.create_cell_list()
    assert g.geometry()["key_max"] < o.geometry()["key_max"]  # fewer, larger cells
    sphgpu.apply(g, sphgpu.reset_rho)
    sphgpu.apply(g, sphgpu.find_rho, self=True)
    if dim == 3 and factor > 1.5:
        with pytest.raises(sphgpu.SphError):
            g.debug_hits()
    else:
        hits = g.debug_hits()
        key = lambda a: a[np.lexsort((a[:, 1], a[:, 0]))]
        assert hits.shape == ref.shape
        assert np.array_equal(key(hits), key(ref))
    g.close()

    g = sphgpu.ParticleSystem(params, sphgpu.MIXED)
    g.upload(c.x, c.v, type=c.type)
    o = oracle_mod.from_case(c)
    g.init_state()
    o.init_state()
    s = o.state()
    fl = s["type"] == G.FLUID
    assert (np.abs(s["rho"] - g.get("rho"))[fl] / s["rho"][fl]).max() <= 1e-6
    assert np.abs(s["P"] - g.get("P")).max() / np.abs(s["P"]).max() <= 2e-6
    assert np.linalg.norm(s["a"] - g.get("a")) / np.linalg.norm(s["a"]) <= 5e-6
    g.close()


def test_cell_factor_limits(gpu):
    """FP64 systems keep the reference's cells; mixed ones accept 1..2."""
    c = G.dam_break(2, 0.05)
    with pytest.raises(sphgpu.SphError):
        sphgpu.ParticleSystem(dict(c.params, cell_factor=1.25), sphgpu.FP64)
    for bad in (0.5, 2.5):
        with pytest.raises(sphgpu.SphError):
            sphgpu.ParticleSystem(dict(c.params, cell_factor=bad), sphgpu.MIXED)
    sphgpu.ParticleSystem(dict(c.params, cell_factor=1.0), sphgpu.FP64).close()


@pytest.mark.parametrize("dim,dr", [(2, 0.02), (3, 0.05)])
def test_mixed_grid_geometry(gpu, dim, dr):
    """A mixed system's cells (cell factor 1): the reference's grid offset by
    5/16 of a cell along each of its axes, the index floor((x - s) / h) taken
    as a product with 1/h, and sph_geometry reports that grid; an FP64
    system keeps the reference's floor(x / h).  On the 3D dam break's lattice
    (h = 4 dr) no particle lies within a fifth of a spacing of a mixed cell's
    boundary, where the reference's grid has whole planes on them."""
    c = G.dam_break(dim, dr)
    p = c.params
    H = p["h"]
    s = [H * (5.0 / 16.0) if d < dim else 0.0 for d in range(3)]
    ic = 1.0 / H
    phase = [int(np.floor((p["domain_min"][d] - s[d]) * ic)) for d in range(3)]
    lim = [int(np.floor((p["domain_max"][d] - s[d]) * ic)) - phase[d] + 1 for d in range(3)]
    g = sphgpu.ParticleSystem(p, sphgpu.MIXED)
    f64 = sphgpu.ParticleSystem(p, sphgpu.FP64)
    try:
        geo = g.geometry()
        assert list(geo["key_phase"]) == phase
        assert list(geo["key_lim"]) == lim
        assert geo["key_max"] == lim[0] * lim[1] * lim[2]
        ref = f64.geometry()
        assert list(ref["key_phase"]) == [int(np.floor(p["domain_min"][d] / H)) for d in range(3)]
        if dim == 3:
            u = (c.x - np.array(s)) * ic
            frac = u - np.floor(u)
            gap = np.minimum(frac, 1.0 - frac) * (H / dr)  # in lattice spacings
            assert gap.min() >= 0.2
            v = c.x / H
            on_boundary = np.abs(v - np.round(v)) * (H / dr) < 1e-6
            assert on_boundary.any()  # the reference's grid: planes on its boundaries
    finally:
        g.close()
        f64.close()
