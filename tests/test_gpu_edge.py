"""Edge cases of the drop-in path against the oracle: an empty system, a
single particle, every particle removed by the binning (NaN and escaped
positions, core.jl:57-70), and pairs placed a few ulps either side of the
support (the FP32 classification band and the reference's exact test,
core.jl:105).  FP64: exact equality of every field and of the ordered pair
list.  Mixed: the same particle count and pair set as FP64, fields within
the mixed path's per-field bounds (density 1e-6 relative)."""
import numpy as np
import pytest

import sphgpu
from sphgpu import geometry as G

pytestmark = pytest.mark.gpu

FIELDS = ("x", "v", "a", "xsph", "rho", "rho_ref", "P")


def _params(dim, H=0.1, hi=1.0, n=1):
    rho0, c0 = 1000.0, 20.0
    g = [0.0, -9.81, 0.0] if dim == 2 else [0.0, 0.0, -9.81]
    return dict(dim=dim, h=H, domain_min=[0.0, 0.0, 0.0],
                domain_max=[hi, hi, hi if dim == 3 else 0.0],
                mass=rho0 * (H / 4.0) ** dim, rho0=rho0, c0=c0, h_smooth=0.5 * H,
                alpha=0.05, eps_xsph=0.5, gravity=g, dt=(0.05 * H) / c0,
                col_height=0.5 * hi, vertical_axis=dim - 1)


def _same(g, o):
    st = o.state()
    assert g.n == o.n
    assert np.array_equal(g.get("oid"), st["oid"])
    for f in FIELDS:
        assert np.array_equal(g.get(f), st[f]), f


def _run_both(c, oracle_mod, steps=3):
    g = sphgpu.ParticleSystem(c.params, sphgpu.FP64)
    g.upload(c.x, c.v, type=c.type)
    o = oracle_mod.from_case(c)
    g.create_cell_list()
    o.create_cell_list()
    assert np.array_equal(g.get("key"), o.keys())
    assert np.array_equal(g.debug_pairs(), o.pairs())
    assert g.pair_count(reset=True) == 0
    g.init_state()
    assert g.pair_count(reset=True) == o.init_state()
    _same(g, o)
    for _ in range(steps):
        g.step(1)
        assert g.pair_count(reset=True) == o.step(1)
    _same(g, o)
    g.synchronize()
    return g, o


@pytest.mark.parametrize("dim", [2, 3])
def test_empty_system(gpu, oracle_mod, dim):
    c = G.Case("empty", dim, 0.025, np.zeros((0, 3)), np.zeros(0, np.int32), np.zeros((0, 3)),
               _params(dim))
    g, o = _run_both(c, oracle_mod)
    assert g.n == 0 and g.get("x").shape == (0, 3) and g.get("rho").shape == (0,)
    gm = sphgpu.ParticleSystem(c.params, sphgpu.MIXED)
    gm.upload(c.x, c.v, type=c.type)
    gm.init_state()
    gm.step(2)
    assert gm.n == 0 and gm.pair_count() == 0
    gm.synchronize()


@pytest.mark.parametrize("dim", [2, 3])
def test_single_particle(gpu, oracle_mod, dim):
    x = np.zeros((1, 3))
    x[0, :dim] = 0.37
    v = np.zeros((1, 3))
    v[0, 0] = 0.25
    c = G.Case("single", dim, 0.025, x, np.zeros(1, np.int32), v, _params(dim))
    g, o = _run_both(c, oracle_mod, steps=4)
    assert g.debug_pairs().shape == (0, 2)
    gm = sphgpu.ParticleSystem(c.params, sphgpu.MIXED)
    gm.upload(c.x, c.v, type=c.type)
    gm.init_state()
    gm.step(4)
    assert gm.pair_count() == 0
    np.testing.assert_allclose(gm.get("rho"), g.get("rho"), rtol=1e-12)
    np.testing.assert_allclose(gm.get("x"), g.get("x"), rtol=1e-12)


@pytest.mark.parametrize("precision", [sphgpu.FP64, sphgpu.MIXED])
def test_every_particle_removed(gpu, oracle_mod, precision):
    c = G.dam_break(2, 0.05)
    x = c.x.copy()
    half = c.n // 2
    x[:half, 0] = np.nan
    x[half:, 1] = -5.0  # below the bounding box
    c.x = x
    g = sphgpu.ParticleSystem(c.params, precision)
    g.upload(c.x, c.v, type=c.type)
    o = oracle_mod.from_case(c)
    g.create_cell_list()
    o.create_cell_list()
    assert g.n == o.n == 0
    g.init_state()
    o.init_state()
    g.step(2)
    o.step(2)
    assert g.n == o.n == 0
    assert g.pair_count() == 0
    g.synchronize()


def _band_case(dim, seed):
    """Targets with neighbours at H (1 + j 2^-52), j = -4..4, along every axis
    and along a diagonal, plus a few random particles; fluid and walls."""
    rng = np.random.default_rng(seed)
    H = 0.1
    centre = np.array([0.5, 0.5, 0.5 if dim == 3 else 0.0])
    pts = [centre.copy()]
    eps = 2.0 ** -52
    dirs = [np.eye(3)[d] for d in range(dim)]
    diag = np.zeros(3)
    diag[:dim] = 1.0 / np.sqrt(dim)
    dirs.append(diag)
    for e in dirs:
        for sgn in (1.0, -1.0):
            for j in range(-4, 5):
                pts.append(centre + sgn * H * (1.0 + j * eps) * e)
    x = np.array(pts)
    extra = rng.uniform(0.3, 0.7, (40, 3))
    if dim == 2:
        extra[:, 2] = 0.0
    x = np.concatenate([x, extra])
    n = x.shape[0]
    typ = np.where(rng.uniform(size=n) < 0.25, G.WALL, G.FLUID).astype(np.int32)
    typ[0] = G.FLUID
    v = np.zeros((n, 3))
    v[:, :dim] = rng.normal(0.0, 0.01, (n, dim))
    v[typ == G.WALL] = 0.0
    return G.Case(f"band_{dim}d", dim, H / 4.0, x, typ, v, _params(dim, H=H))


@pytest.mark.parametrize("dim", [2, 3])
def test_pairs_at_the_support_edge(gpu, oracle_mod, dim):
    c = _band_case(dim, 11 + dim)
    g, o = _run_both(c, oracle_mod, steps=2)
    # the mixed path classifies with the same FP32 band and exact test
    g2 = sphgpu.ParticleSystem(c.params, sphgpu.FP64)
    gm = sphgpu.ParticleSystem(c.params, sphgpu.MIXED)
    for s in (g2, gm):
        s.upload(c.x, c.v, type=c.type)
        s.init_state()
    assert gm.pair_count(reset=True) == g2.pair_count(reset=True)
    sm, s64 = gm.pair_stats(), g2.pair_stats()
    for cat in ("density", "wall", "force_fluid", "force_wall"):
        assert sm[cat] == s64[cat], cat
    np.testing.assert_allclose(gm.get("rho"), g2.get("rho"), rtol=1e-6)
