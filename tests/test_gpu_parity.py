"""FP64 GPU path against the CPU oracle: bit-exact cell keys, neighbour-pair
lists (order included), fields after every operator, after the initial state
and after many steps; removal semantics; sums; the collision test of
tests/test_collision_2d.jl on the GPU.

Tolerance: the FP64 path is compiled without FMA contraction and evaluates
every expression in the oracle's order, so the comparison is exact equality
(any difference fails; 1e-12 relative per step is the stated bar)."""
import math

import numpy as np
import pytest

import sphgpu
from sphgpu import geometry as G

pytestmark = pytest.mark.gpu

FIELDS = ("x", "v", "a", "xsph", "rho", "rho_ref", "P")


def make(case, oracle_mod, precision=sphgpu.FP64):
    g = sphgpu.ParticleSystem(case.params, precision)
    g.upload(case.x, case.v, type=case.type)
    o = oracle_mod.from_case(case)
    return g, o


def assert_same_state(g, o, fields=FIELDS):
    st = o.state()
    assert g.n == o.n
    assert np.array_equal(g.get("oid"), st["oid"])
    assert np.array_equal(g.get("type"), st["type"])
    for f in fields:
        a, b = g.get(f), st[f]
        if not np.array_equal(a, b):
            bad = np.argwhere(a != b)
            i = bad[0][0]
            raise AssertionError(f"field {f} differs at {len(bad)} entries; first {i}: "
                                 f"gpu {a[i]!r} oracle {b[i]!r}")


@pytest.mark.parametrize("dim,dr", [(2, 0.02), (3, 0.05)])
def test_keys_and_pairs_bitexact(gpu, oracle_mod, dim, dr):
    c = G.dam_break(dim, dr)
    g, o = make(c, oracle_mod)
    assert g.geometry() == o.geometry()
    g.create_cell_list()
    o.create_cell_list()
    assert np.array_equal(g.get("key"), o.keys())
    gp, op = g.debug_pairs(), o.pairs()
    assert gp.shape == op.shape
    assert np.array_equal(gp, op)


@pytest.mark.parametrize("dim,dr,steps", [(2, 0.02, 30), (3, 0.05, 5)])
def test_init_and_steps_bitexact(gpu, oracle_mod, dim, dr, steps):
    c = G.dam_break(dim, dr)
    g, o = make(c, oracle_mod)
    g.init_state()
    p_o = o.init_state()
    assert g.pair_count(reset=True) == p_o
    assert_same_state(g, o)
    for _ in range(steps):
        g.step(1)
        p_o = o.step(1)
        assert g.pair_count(reset=True) == p_o
    assert_same_state(g, o)
    g.synchronize()


def test_reference_style_operator_sequence(gpu, oracle_mod):
    """apply!/apply_unary! one operator at a time, as a user time loop calls them."""
    c = G.dam_break(2, 0.04)
    g, o = make(c, oracle_mod)
    for sysm in (g, o):
        sysm.create_cell_list()
    ops = [(sphgpu.reset_rho0, None), (sphgpu.find_rho0, True), (sphgpu.hydrostatic, None),
           (sphgpu.reset_rho, None), (sphgpu.find_rho, True), (sphgpu.find_pressure, None),
           (sphgpu.wall_pressure, False), (sphgpu.reset_a, None),
           (sphgpu.internal_force, False), (sphgpu.accelerate, None),
           (sphgpu.move, None)]
    for op, self_term in ops:
        sphgpu.apply(g, op, self=bool(self_term))
        if op.binary:
            o.apply(op.op, bool(self_term))
        else:
            o.apply_unary(op.op)
    assert_same_state(g, o)
    # move! leaves the cell list stale: a pair pass must be refused
    with pytest.raises(sphgpu.SphError):
        sphgpu.apply(g, sphgpu.find_rho, self=True)
    g.create_cell_list()
    o.create_cell_list()
    sphgpu.apply(g, sphgpu.internal_force)
    o.apply(sphgpu.internal_force.op, False)
    assert_same_state(g, o)


@pytest.mark.parametrize("dim,dr", [(2, 0.04), (3, 0.08)])
def test_fields_set_between_passes(gpu, oracle_mod, dim, dr):
    """Velocities, densities and pressures set through ParticleField between
    the density and force passes of one binning: the force pass sees the new
    values (the FP64 force pass rebuilds its particle records from the
    fields), bit for bit as the oracle."""
    c = G.dam_break(dim, dr)
    g, o = make(c, oracle_mod)
    g.init_state()
    o.init_state()
    rng = np.random.default_rng(dim)
    for sysm in (g, o):
        sysm.create_cell_list()
    sphgpu.apply(g, sphgpu.reset_rho)
    o.apply_unary(sphgpu.reset_rho.op)
    sphgpu.apply(g, sphgpu.find_rho, self=True)
    o.apply(sphgpu.find_rho.op, True)
    st = o.state()
    v = st["v"].copy()
    v[:, :dim] += rng.normal(0.0, 0.05, (c.n, dim))
    v[st["type"] == G.WALL] = 0.0
    rho = st["rho"] * (1.0 + rng.uniform(-1e-3, 1e-3, c.n))
    g.set("v", v)
    g.set("rho", rho)
    o.set_state(v=v, rho=rho)
    for sysm_ops in ((sphgpu.find_pressure, None), (sphgpu.wall_pressure, False),
                     (sphgpu.reset_a, None), (sphgpu.internal_force, False)):
        op, self_term = sysm_ops
        sphgpu.apply(g, op, self=bool(self_term))
        if op.binary:
            o.apply(op.op, bool(self_term))
        else:
            o.apply_unary(op.op)
    assert_same_state(g, o)
    # and once more with only v changed after the EOS and the wall pressure
    v2 = v.copy()
    v2[:, 0] *= 0.5
    g.set("v", v2)
    o.set_state(v=v2)
    sphgpu.apply(g, sphgpu.reset_a)
    o.apply_unary(sphgpu.reset_a.op)
    sphgpu.apply(g, sphgpu.internal_force)
    o.apply(sphgpu.internal_force.op, False)
    assert_same_state(g, o)


def test_removal_tail_fill_bitexact(gpu, oracle_mod):
    c = G.dam_break(2, 0.05)
    rng = np.random.default_rng(7)
    x = c.x.copy()
    out = rng.choice(c.n, 40, replace=False)
    x[out[:20], 0] = np.nan
    x[out[20:30], 1] = 100.0
    x[out[30:], 0] = -1.0
    c.x = x
    g, o = make(c, oracle_mod)
    g.create_cell_list()
    o.create_cell_list()
    assert g.n == o.n == c.n - 40
    assert_same_state(g, o, fields=("x", "v", "rho"))
    assert np.array_equal(g.get("key"), o.keys())
    assert np.array_equal(g.debug_pairs(), o.pairs())
    # and the dynamics continue identically
    g.init_state()
    o.init_state()
    g.step(3)
    o.step(3)
    assert_same_state(g, o)


def test_removal_during_steps(gpu, oracle_mod):
    """Particles pushed out of the bounding box by the drift are removed in the
    step's binning exactly as create_cell_list! removes them."""
    c = G.dam_break(2, 0.05)
    v = np.zeros_like(c.x)
    fluid = np.nonzero(c.type == 0)[0]
    v[fluid[-30:], 1] = 5.0e3  # leaves through the open top within a step or two
    c.v = v
    g, o = make(c, oracle_mod)
    g.init_state()
    o.init_state()
    for _ in range(4):
        g.step(1)
        o.step(1)
    assert o.n < c.n
    assert_same_state(g, o)


def test_sums_bitexact(gpu, oracle_mod):
    c = G.dam_break(2, 0.04)
    g, o = make(c, oracle_mod)
    g.init_state()
    o.init_state()
    rng = np.random.default_rng(3)
    pts = np.zeros((500, 3))
    pts[:, 0] = rng.uniform(-0.5, 4.5, 500)
    pts[:, 1] = rng.uniform(-0.5, 3.5, 500)
    pts[0] = [math.nan, 0.0, 0.0]
    pts[1] = [0.5, 1.0, 0.3]  # off the 2D plane
    pts[2] = [1e300, 0.0, 0.0]
    for f, of in ((sphgpu.DENSITY, oracle_mod.SUM_DENSITY), (sphgpu.KERNEL, oracle_mod.SUM_KERNEL),
                  (sphgpu.PRESSURE, oracle_mod.SUM_PRESSURE), (sphgpu.SHEPARD, oracle_mod.SUM_SHEPARD)):
        a = sphgpu.sum(g, f, pts)
        b = o.sum_points(of, pts)
        assert np.array_equal(a, b, equal_nan=True)
        idx = rng.choice(c.n, 200, replace=False)
        a = sphgpu.sum(g, f, particles=idx)
        b = o.sum_particles(of, idx)
        assert np.array_equal(a, b)


def test_collision_2d_as_written_gpu(gpu, oracle_mod):
    """tests/test_collision_2d.jl run as written (its scenario, linear EOS,
    P/rho0^2 pressure force, no gravity, its initialisation and time loop to
    t = 1.0, 4,168 steps) on the GPU and on the oracle: every field equal to
    the oracle's bit for bit at each of the test's ten records and at the
    end, and the test's own assertions on the GPU's records -- a constant
    particle count and a relative energy increase below 1e-2."""
    from test_oracle_collision import initialise, run_collision
    c = G.collision_2d()
    g, o = make(c, oracle_mod)
    initialise(g.create_cell_list, lambda op, s: sphgpu.apply(g, sphgpu.op_by_id(op), self=s),
               lambda op: sphgpu.apply(g, sphgpu.op_by_id(op)))
    initialise(o.create_cell_list, o.apply, o.apply_unary)
    assert_same_state(g, o)
    records = []

    def step_both(k):
        g.step(k)
        o.step(k)

    def check(k, st):
        records.append(k)
        assert_same_state(g, o)

    N, E = run_collision(step_both, lambda: {f: g.get(f) for f in ("v", "rho", "rho_ref")},
                         lambda: g.n, c.params, on_record=check)
    assert records == [417 * j for j in range(10)]
    assert_same_state(g, o)
    assert np.all(N == N[0])
    assert np.max(E / E[0] - 1.0) < 1e-2
    g.synchronize()


def test_large_2d_first_steps_bitexact(gpu, oracle_mod):
    """The 1.0M-particle 2D dam break (dr = 0.0014), checked against the CPU
    restatement on its first 5 steps."""
    c = G.dam_break(2, 0.0014)
    g, o = make(c, oracle_mod)
    g.init_state()
    o.init_state()
    g.step(5)
    o.step(5)
    assert_same_state(g, o, fields=("x", "v", "rho", "P", "a"))


def test_long_rows_bitexact(gpu, oracle_mod):
    """3D dam break with H = 4.6 dr: interior targets have ~400 neighbours
    per row (rows are sized from the counts, so they hold them)."""
    c = G.dam_break(3, 0.1, h_factor=2.3)
    g, o = make(c, oracle_mod)
    g.init_state()
    assert g.pair_count(reset=True) == o.init_state()
    assert_same_state(g, o)
    for _ in range(3):
        g.step(1)
        assert g.pair_count(reset=True) == o.step(1)
    assert_same_state(g, o)
    g.synchronize()


def test_row_segment_overflow_bitexact(gpu, oracle_mod):
    """1,000 fluid and 500 wall particles inside one cell, all within H of one
    another: every fluid row has a segment of 1,499 neighbours, more than a
    10-bit rank addresses (1,022), so every row is marked overflowed and
    every target takes the traversal."""
    rng = np.random.default_rng(3)
    nf, nw = 1000, 500
    n = nf + nw
    H = 0.1
    x = 0.52 + rng.uniform(0.0, 0.05, (n, 3))
    typ = np.concatenate([np.full(nf, G.FLUID, np.int32), np.full(nw, G.WALL, np.int32)])
    v = np.zeros((n, 3))
    v[:nf] = rng.normal(0.0, 0.01, (nf, 3))
    rho0, c0 = 1000.0, 20.0
    params = dict(dim=3, h=H, domain_min=[0.0, 0.0, 0.0], domain_max=[1.0, 1.0, 1.0],
                  mass=rho0 * 0.05 ** 3 / n, rho0=rho0, c0=c0, h_smooth=0.5 * H, alpha=0.05,
                  eps_xsph=0.5, gravity=[0.0, 0.0, -9.81], dt=(0.05 * H) / c0,
                  col_height=0.6, vertical_axis=2)
    c = G.Case("cluster", 3, H / 4.0, x, typ, v, params)
    g, o = make(c, oracle_mod)
    g.init_state()
    assert g.pair_count(reset=True) == o.init_state()
    assert_same_state(g, o)
    for _ in range(2):
        g.step(1)
        assert g.pair_count(reset=True) == o.step(1)
    assert_same_state(g, o)
    g.synchronize()


@pytest.mark.parametrize("dim,dr", [(2, 0.04), (3, 0.08)])
def test_rows_grow_when_the_flow_needs_more(gpu, oracle_mod, dim, dr):
    """The FP64 rows are sized from the counts of the first density pass
    (which traverses, having none).  A flow that packs its particles closer
    needs more entries than the rows hold: that pass traverses instead
    (results unchanged), reports the shortfall, and the rows grow before
    the next pass -- inside sph_step's captured step graph too, which is then
    captured again.  Bit-exact with the oracle throughout."""
    c = G.dam_break(dim, dr)
    g, o = make(c, oracle_mod)
    g.init_state()
    assert g.pair_count(reset=True) == o.init_state()
    used0 = g.memory_usage()
    st = o.state()
    x = st["x"].copy()
    fl = st["type"] == G.FLUID
    x0 = x[fl, :dim].min(axis=0)
    x[fl, :dim] = x0 + 0.85 * (x[fl, :dim] - x0)  # about 1/0.85^dim the neighbours
    g.set("x", x)
    o.set_state(x=x)
    g.step(1)  # its density pass overflows and traverses
    assert g.pair_count(reset=True) == o.step(1)
    assert_same_state(g, o)
    g.step(6)  # the step graph: the rows grow first, then it is captured again
    assert g.pair_count(reset=True) == o.step(6)
    assert_same_state(g, o)
    assert g.memory_usage() > used0
    g.synchronize()


def _narrow_case(dim, n, seed):
    """Random fluid and wall particles in a domain one cell wide along x
    (and two along y in 3D): key + key_diff wraps between rows of cells and
    reaches the same cell through several slots, which the reference's
    range test (core.jl:98) keeps, so pairs repeat."""
    rng = np.random.default_rng(seed)
    H = 0.1
    if dim == 2:
        hi = [0.9 * H, 10.0 * H, 0.0]
    else:
        hi = [0.9 * H, 1.9 * H, 4.0 * H]
    x = np.zeros((n, 3))
    for d in range(dim):
        x[:, d] = rng.uniform(0.0, hi[d], n)
    typ = np.where(rng.uniform(size=n) < 0.2, G.WALL, G.FLUID).astype(np.int32)
    v = np.zeros((n, 3))
    v[:, :dim] = rng.normal(0.0, 0.05, (n, dim))
    v[typ == G.WALL] = 0.0
    rho0, c0 = 1000.0, 20.0
    vol = np.prod(hi[:dim]) / n
    params = dict(dim=dim, h=H, domain_min=[0.0, 0.0, 0.0], domain_max=hi, mass=rho0 * vol,
                  rho0=rho0, c0=c0, h_smooth=0.5 * H, alpha=0.05, eps_xsph=0.5,
                  gravity=[0.0, -9.81, 0.0] if dim == 2 else [0.0, 0.0, -9.81],
                  dt=(0.05 * H) / c0, col_height=hi[dim - 1], vertical_axis=dim - 1)
    return G.Case(f"narrow_{dim}d_{n}", dim, H / 4.0, x, typ, v, params)


@pytest.mark.parametrize("dim,n", [(2, 150), (2, 400), (3, 300)])
def test_wrapped_cells_bitexact(gpu, oracle_mod, dim, n):
    c = _narrow_case(dim, n, 7 + n)
    g, o = make(c, oracle_mod)
    assert g.geometry()["key_lim"][0] == 1  # one cell along x
    g.init_state()
    assert g.pair_count(reset=True) == o.init_state()
    assert_same_state(g, o)
    for _ in range(3):
        g.step(1)
        assert g.pair_count(reset=True) == o.step(1)
    assert_same_state(g, o)
    g.synchronize()


def test_bad_arguments_raise(gpu):
    c = G.dam_break(2, 0.1)
    g = sphgpu.ParticleSystem(c.params)
    x = c.x.copy()
    x[0, 2] = 1.0
    with pytest.raises(sphgpu.SphError):
        g.upload(x, type=c.type)
    g.upload(c.x, type=c.type)
    with pytest.raises(sphgpu.SphError):
        g.apply(sphgpu.Operator("bogus", 99, True))
    with pytest.raises(sphgpu.SphError):  # cells never built
        g.apply(sphgpu.find_rho, True)
    with pytest.raises(sphgpu.SphError):
        g.sum_particles(sphgpu.DENSITY, [c.n + 5])
