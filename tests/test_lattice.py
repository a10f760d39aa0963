"""Particle counts of the dam-break lattices under the reference's lattice
rules (grids.jl:52-66, :128-144; geometry.jl:24-43, :198-234)."""
import pytest

from sphgpu import geometry as G


@pytest.mark.parametrize("dim,dr,lid,fluid,walls", [
    (2, 0.02, True, 5151, 1977),
    (2, 0.02, False, 5151, 1361),
    (2, 0.0014, False, 1021735, 21440),
])
def test_dam_break_counts_2d(dim, dr, lid, fluid, walls):
    c = G.dam_break(dim, dr, lid=lid)
    assert c.n_fluid == fluid
    assert c.n - c.n_fluid == walls


def test_dam_break_counts_3d():
    c = G.dam_break(3, 0.0079)
    assert c.n_fluid == 4096766
    assert c.n - c.n_fluid == 1649867


def test_order_is_reference_loop_order():
    # covering() loops i outer, j inner: x changes slowest
    c = G.dam_break(2, 0.25)
    xf = c.x[: c.n_fluid]
    assert (xf[1, 0], xf[1, 1]) == (0.0, 0.25)
    assert xf[0, 0] == xf[8, 0] and xf[9, 0] == 0.25


def test_collision_circles():
    c = G.collision_2d()
    # two mirror-image circles: equal halves
    assert c.n % 2 == 0
    assert (c.v[: c.n // 2, 0] == 1.0).all() and (c.v[c.n // 2:, 0] == -1.0).all()
