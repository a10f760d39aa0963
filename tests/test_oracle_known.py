"""Known-answer tests of the oracle, derived by hand from the reference source.

structs.jl:57-106 (cell-key geometry, find_key), core.jl:51-90 (removal,
tail-fill compaction, descending cells), core.jl:94-161 (traversal, self term
last), core.jl:240-291 (sums include every particle within h).
"""
import math
from fractions import Fraction

import numpy as np
import pytest

from sphgpu import geometry as G


def params2d(h=0.096, lo=(-0.06, -0.06), hi=(4.06, 3.06)):
    return dict(dim=2, h=h, domain_min=[lo[0], lo[1], 0.0], domain_max=[hi[0], hi[1], 0.0],
                mass=1.0, rho0=1000.0, c0=10.0, h_smooth=h / 2, alpha=0.0, eps_xsph=0.0,
                gravity=[0.0, 0.0, 0.0], dt=1e-4, col_height=0.0, vertical_axis=1)


def test_geometry_2d(oracle_mod):
    s = oracle_mod.OracleSystem(params2d())
    g = s.geometry()
    # floor(-0.06/0.096) = -1; floor(4.06/0.096) = 42 -> 42+1+1; floor(3.06/0.096) = 31
    assert g["key_phase"] == (-1, -1, 0)
    assert g["key_lim"] == (44, 33, 1)
    assert g["key_max"] == 44 * 33
    # structs.jl:73-75: for di in -1:1, dj in -1:1 -> di + L1*dj, di outermost
    assert g["key_diff"] == [-45, -1, 43, -44, 0, 44, -43, 1, 45]


def test_geometry_3d(oracle_mod):
    p = params2d(h=0.3)
    p.update(dim=3, domain_min=[0.0, 0.0, 0.0], domain_max=[1.0, 1.0, 1.0], vertical_axis=2)
    s = oracle_mod.OracleSystem(p)
    g = s.geometry()
    assert g["key_phase"] == (0, 0, 0)
    assert g["key_lim"] == (4, 4, 4)
    assert g["key_max"] == 64
    # structs.jl:79-81: di outer, dj middle, dk inner: di + 4*(dj + 4*dk)
    assert g["key_diff"][:4] == [-21, -5, 11, -17]
    assert g["key_diff"][13] == 0
    assert g["key_diff"][-1] == 21
    assert len(g["key_diff"]) == 27


def test_find_key(oracle_mod):
    s = oracle_mod.OracleSystem(params2d())
    # i = 1 + floor(x/h) - key_phase: (0,0) -> (2, 2, 1) -> 2 + 44*1
    assert s.find_key((0.0, 0.0, 0.0)) == 46
    # (0.1, 0.2): floor(1.04) = 1 -> i = 3; floor(2.08) = 2 -> j = 4 -> 3 + 44*3
    assert s.find_key((0.1, 0.2, 0.0)) == 135
    # Int64(floor(NaN)) and Int64(floor(Inf)) throw -> -1 (structs.jl:103-105)
    assert s.find_key((math.nan, 0.0, 0.0)) == -1
    assert s.find_key((0.0, math.inf, 0.0)) == -1
    assert s.find_key((1e300, 0.0, 0.0)) == -1


def _line_system(oracle_mod, n=10):
    s = oracle_mod.OracleSystem(params2d(h=0.5, lo=(0.0, 0.0), hi=(10.0, 1.0)))
    x = np.zeros((n, 3))
    x[:, 0] = np.arange(n) + 0.25
    x[:, 1] = 0.5
    return s, x


@pytest.mark.parametrize("removed,expected", [
    # 1-based removal sets and the survivors' original 1-based indices after
    # particles[removal[i]] = particles[end+1-i] in descending removal order
    ({3, 9}, [1, 2, 10, 4, 5, 6, 7, 8]),
    ({8, 10}, [1, 2, 3, 4, 5, 6, 7, 9]),
    ({7, 8, 10}, [1, 2, 3, 4, 5, 6, 9]),
    ({1}, [10, 2, 3, 4, 5, 6, 7, 8, 9]),
    ({1, 2, 3, 4, 5, 6, 7, 8, 9, 10}, []),
])
def test_removal_tail_fill(oracle_mod, removed, expected):
    s, x = _line_system(oracle_mod)
    for r in removed:
        x[r - 1, 0] = math.nan if r % 2 else 50.0  # NaN or outside the box
    s.add_particles(x)
    s.create_cell_list()
    assert s.n == len(expected)
    assert list(s.state()["oid"] + 1) == expected


def test_descending_cell_order_and_self_last(oracle_mod):
    # target 0 and three neighbours in one cell: the pair list visits them in
    # descending index order (core.jl:31-37 keeps cells descending)
    s = oracle_mod.OracleSystem(params2d(h=1.0, lo=(0.0, 0.0), hi=(3.0, 3.0)))
    x = np.array([[1.5, 1.5, 0.0], [1.2, 1.2, 0.0], [1.7, 1.4, 0.0], [1.1, 1.8, 0.0]])
    s.add_particles(x)
    s.create_cell_list()
    pairs = s.pairs()
    assert [tuple(p) for p in pairs[pairs[:, 0] == 0]] == [(0, 3), (0, 2), (0, 1)]
    assert [tuple(p) for p in pairs[pairs[:, 0] == 2]] == [(2, 3), (2, 1), (2, 0)]


def test_two_particle_density_exact(oracle_mod):
    """rho_p = m W(r) + m W(0) (neighbour, then the self term), against the
    closed form of wendland2 in rationals."""
    h = 0.25
    p = params2d(h=h, lo=(0.0, 0.0), hi=(1.0, 1.0))
    p["mass"] = 0.37
    s = oracle_mod.OracleSystem(p)
    x = np.array([[0.5, 0.5, 0.0], [0.5 + 0.1, 0.5 + 0.05, 0.0]])
    s.add_particles(x, type=np.zeros(2, np.int32))
    s.create_cell_list()
    s.apply_unary(oracle_mod.OP_RESET_RHO)
    pairs = s.apply(oracle_mod.OP_DENSITY, True)
    assert pairs == 2
    rho = s.state()["rho"]
    d = Fraction(float(x[1, 0])) - Fraction(float(x[0, 0]))
    e = Fraction(float(x[1, 1])) - Fraction(float(x[0, 1]))
    r = math.sqrt(float(d * d + e * e))
    C = Fraction(2.228169203286535)
    H = Fraction(h)
    m = Fraction(0.37)
    xr = Fraction(r) / H
    w = C * (1 - xr) ** 4 * (1 + 4 * xr) / H ** 2
    w0 = C / H ** 2
    assert rho[0] == pytest.approx(float(m * w + m * w0), rel=4e-15)
    assert rho[0] == rho[1]


def test_sums_include_every_particle(oracle_mod):
    c = G.dam_break(2, 0.1)
    s = oracle_mod.from_case(c)
    s.create_cell_list()
    s.apply_unary(oracle_mod.OP_RESET_RHO)
    s.apply(oracle_mod.OP_DENSITY, True)
    st = s.state()
    fluid = np.nonzero(st["type"] == 0)[0][:50]
    # sum(sys, func, p) includes p itself (core.jl:271-291): equals rho up to
    # summation order
    got = s.sum_particles(oracle_mod.SUM_DENSITY, fluid)
    np.testing.assert_allclose(got, st["rho"][fluid], rtol=1e-13)
    # a point far outside every cell sums to zero
    assert s.sum_points(oracle_mod.SUM_DENSITY, [[100.0, 100.0, 0.0]])[0] == 0.0


def test_stale_cells_refused(oracle_mod):
    c = G.dam_break(2, 0.1)
    s = oracle_mod.from_case(c)
    s.create_cell_list()
    s.apply_unary(oracle_mod.OP_DRIFT)
    with pytest.raises(RuntimeError):
        s.apply(oracle_mod.OP_DENSITY, True)


def test_result_independent_of_threads(oracle_mod):
    """core.jl:126 threads over targets only; the oracle's OpenMP split must
    not change any bit (checked against a 2-step run; thread count is set by
    OMP_NUM_THREADS in a child process)."""
    import subprocess
    import sys
    code = (
        "import sys; sys.path[:0] = {paths!r}\n"
        "import numpy as np, oracle as O\n"
        "from sphgpu import geometry as G\n"
        "c = G.dam_break(2, 0.05); s = O.from_case(c); s.init_state(); s.step(2)\n"
        "st = s.state(); np.save(sys.argv[1], np.concatenate([st['x'].ravel(), st['rho']]))\n")
    import os
    import tempfile
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    paths = [root, os.path.join(root, "smoothedparticles.jl_gb300"), os.path.join(root, "oracle")]
    outs = []
    with tempfile.TemporaryDirectory() as td:
        for nt in (1, 3):
            f = os.path.join(td, f"o{nt}.npy")
            env = dict(os.environ, OMP_NUM_THREADS=str(nt))
            subprocess.run([sys.executable, "-c", code.format(paths=paths), f], env=env, check=True)
            outs.append(np.load(f))
    assert np.array_equal(outs[0], outs[1])
