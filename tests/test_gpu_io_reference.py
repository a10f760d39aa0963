"""tests/test_IO.jl restated: a particle system in the circle of radius 1
(dr = 1/100, ParticleSystem h = 0.1), whose particles carry data that are
functions of their position (s = x2, v = x2 e_x - x1 e_y; get_vars), is saved
as one frame (new_pvd_file, save_frame!, save_pvd_file: "save data to vtk")
and imported into a fresh system twice (import_particles!: "read data from
vtk"): the frame and the collection exist, the first import reproduces the
particle count and every value exactly, the second doubles the count with the
same data.

Differences from the test as written: the points are the square lattice's
inside the circle (the test's hexagonal grid only places the points; this
library generates square and cubic lattices), the scalar s is carried in the
density field (the system's fields are the built-in ones), and the matrix
field M is not carried (RealMatrix fields are outside this library)."""
import os

import numpy as np
import pytest

import sphgpu
from sphgpu.vtk import import_particles, new_pvd_file, read_pvd, save_frame, save_pvd_file

pytestmark = pytest.mark.gpu

DR = 1 / 100


def circle_points(dr, r=1.0):
    """Lattice points i*dr inside Circle(0, 0, r) (geometry.jl is_inside:
    x1^2 + x2^2 <= r^2), i outer, j inner."""
    i = np.arange(int(np.floor(-r / dr)), int(np.ceil(r / dr)) + 1)
    X, Y = np.meshgrid(i * dr, i * dr, indexing="ij")
    x = np.stack([X.ravel(), Y.ravel(), np.zeros(X.size)], axis=1)
    return x[(x[:, 0] * x[:, 0] + x[:, 1] * x[:, 1]) <= r * r]


def get_vars(x):
    """test_IO.jl get_vars: s = x[2], v = x[2] VECX - x[1] VECY."""
    s = x[:, 1].copy()
    v = np.stack([x[:, 1], -x[:, 0], np.zeros(x.shape[0])], axis=1)
    return s, v


def make_sys():
    """ParticleSystem(Particle, Circle(0, 0, 1), 0.1): the circle's bounding box."""
    params = dict(dim=2, h=0.1, domain_min=[-1.0, -1.0, 0.0], domain_max=[1.0, 1.0, 0.0],
                  mass=1.0, rho0=1.0, c0=1.0, h_smooth=0.05, alpha=0.0, eps_xsph=0.0,
                  gravity=[0.0, 0.0, 0.0], dt=1e-3, col_height=0.0, vertical_axis=1)
    return sphgpu.ParticleSystem(params, sphgpu.FP64)


def test_io_as_in_the_reference(gpu, tmp_path):
    x = circle_points(DR)
    s, v = get_vars(x)
    sys_ = make_sys()
    sys_.upload(x, v, rho=s)
    n = sys_.n
    assert n == x.shape[0]

    # @testset "save data to vtk"
    out = str(tmp_path / "test_IO")
    data = new_pvd_file(sys_, out)
    save_frame(data, "v", "rho")
    save_pvd_file(data)
    assert os.path.isfile(os.path.join(out, "frame0.vtp"))
    assert os.path.isfile(os.path.join(out, "result.pvd"))
    assert [f for _, f in read_pvd(os.path.join(out, "result.pvd"))] == \
        [os.path.join(out, "frame0.vtp")]

    # @testset "read data from vtk"
    imp = make_sys()
    assert import_particles(imp, os.path.join(out, "frame0.vtp")) == n
    assert imp.n == n
    xi = imp.get("x")
    si, vi = get_vars(xi)
    assert np.array_equal(xi, x)
    assert np.array_equal(imp.get("rho"), si)
    assert np.array_equal(imp.get("v"), vi)
    # import even more particles
    assert import_particles(imp, os.path.join(out, "frame0.vtp")) == n
    assert imp.n == 2 * n
    xi = imp.get("x")
    si, vi = get_vars(xi)
    assert np.array_equal(imp.get("rho"), si)
    assert np.array_equal(imp.get("v"), vi)
    assert np.array_equal(xi[n:], x)
    sys_.close()
    imp.close()
