"""Edge cases of the CPU oracle itself: an empty system, a single particle
(its density is the self term m W(0) alone, core.jl:155-157, and no force
acts on it), and every particle removed by create_cell_list! (core.jl:57-70)."""
import numpy as np
import pytest

from sphgpu import geometry as G


def _params(dim, H=0.1):
    rho0, c0 = 1000.0, 20.0
    g = [0.0, -9.81, 0.0] if dim == 2 else [0.0, 0.0, -9.81]
    return dict(dim=dim, h=H, domain_min=[0.0, 0.0, 0.0],
                domain_max=[1.0, 1.0, 1.0 if dim == 3 else 0.0],
                mass=rho0 * (H / 4.0) ** dim, rho0=rho0, c0=c0, h_smooth=0.5 * H,
                alpha=0.05, eps_xsph=0.5, gravity=g, dt=(0.05 * H) / c0,
                col_height=0.5, vertical_axis=dim - 1)


@pytest.mark.parametrize("dim", [2, 3])
def test_empty_system(oracle_mod, dim):
    c = G.Case("empty", dim, 0.025, np.zeros((0, 3)), np.zeros(0, np.int32), np.zeros((0, 3)),
               _params(dim))
    o = oracle_mod.from_case(c)
    o.create_cell_list()
    assert o.n == 0 and o.keys().shape == (0,) and o.pairs().shape == (0, 2)
    assert o.init_state() == 0
    assert o.step(3) == 0
    assert o.state()["x"].shape == (0, 3)


@pytest.mark.parametrize("dim", [2, 3])
def test_single_particle_self_term_only(oracle_mod, dim):
    x = np.zeros((1, 3))
    x[0, :dim] = 0.37
    p = _params(dim)
    c = G.Case("single", dim, 0.025, x, np.zeros(1, np.int32), np.zeros((1, 3)), p)
    o = oracle_mod.from_case(c)
    assert o.init_state() == 0
    h = p["h"]
    cw = 2.228169203286535 / (h * h) if dim == 2 else 3.3422538049298023 / (h * h * h)
    st = o.state()
    assert st["rho"][0] == p["mass"] * cw       # m W(0), W(0) = C_w
    assert np.array_equal(st["a"], np.zeros((1, 3)))
    assert o.step(4) == 0
    assert np.array_equal(o.state()["a"], np.zeros((1, 3)))


def test_every_particle_removed(oracle_mod):
    c = G.dam_break(2, 0.05)
    x = c.x.copy()
    x[: c.n // 2, 0] = np.nan
    x[c.n // 2:, 1] = -5.0
    c.x = x
    o = oracle_mod.from_case(c)
    o.create_cell_list()
    assert o.n == 0
    assert o.init_state() == 0 and o.step(2) == 0
