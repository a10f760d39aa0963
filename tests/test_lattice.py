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


# tests/test_geometry.jl restated for the shapes and grids this library
# generates (square and cubic grids): the covering's particle count times the
# cell area (volume) of a grid of spacing 1/N, N = 200, against the shape's
# area (volume), within the test's tolerances rtol_2d = 0.01, rtol_3d = 0.03
# (test_geometry.jl:6-11, :17-45).  The reference covers the rectangle with
# its hexagonal grid; here it is covered with the square grid.
N = 200


def test_geometry_area_circle():
    x = G.circle(2, 1.0 / N, 0.0, 0.0, 1.0)           # test_geometry.jl:66-68
    assert abs(x.shape[0] / N ** 2 / 3.141592653589793 - 1.0) < 0.01


def test_geometry_area_rectangle():
    x = G.fill_box(2, 1.0 / N, G.rectangle(0.0, -1.0, 2.0, 5.0))  # :70-72
    assert abs(x.shape[0] / N ** 2 / 12.0 - 1.0) < 0.01


def test_geometry_volume_box():
    x = G.fill_box(3, 1.0 / N, G.box3(-0.7, -0.6, -0.5, 0.7, 0.6, 0.5))  # :118-120
    assert abs(x.shape[0] / N ** 3 / (1.4 * 1.2 * 1.0) - 1.0) < 0.03
