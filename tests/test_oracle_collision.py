"""tests/test_collision_2d.jl run as written, on the oracle.

The scenario is the test's own (two circles of radius 0.4, dr = 0.02, kernel
support h = 2.4 dr, c = 20, rho0 = 1000, m = rho0 dr^2, dt = 0.1 h / c,
t_end = 1.0; test_collision_2d.jl:15-58) with its operators: find_rho0! and
find_rho! (density sums with the self term), the linear equation of state
find_pressure! P = c^2 (rho - rho0) (:71-73), internal_force! with the
pressure term P/rho0^2 (:75-78) and accelerate! without gravity (:92-94).
The library's built-ins give exactly these with sph_params.eos =
SPH_EOS_LINEAR, alpha = 0 (no viscosity), eps_xsph = 0 (no XSPH) and zero
gravity; their FP64 evaluation order is the library's (mass folded into the
kernel constants, sums with fused multiply-adds), the same in the oracle
and on the GPU.

The sequence is the test's: the initialisation of main() (:123-127), then
verlet_step! (:106-116) for k = 0 .. round(t_end/dt), recording the particle
count and the energy (:96-100) after every step with k % round(dt_frame/dt)
== 0, and finally its two assertions (:141-147): a constant particle count
and a relative energy increase below 1e-2.
"""
import numpy as np

import oracle
from sphgpu import geometry as G


def collision_schedule(params, t_end=1.0):
    """(steps of the time loop, steps between two records) as the test
    computes them: k = 0 : round(t_end/dt), record when k % round(dt_frame/dt)
    == 0, dt_frame = t_end/10 (test_collision_2d.jl:31-33, 131-133)."""
    dt = params["dt"]
    return int(round(t_end / dt)) + 1, int(round((t_end / 10.0) / dt))


def energy(st, params):
    """test_collision_2d.jl:96-100 summed over the particles: kinetic
    0.5 m v.v plus internal 0.5 m c^2 (rho - rho0_p)^2 / rho0^2, rho0_p the
    particle's own reference density."""
    m, c, rho0 = params["mass"], params["c0"], params["rho0"]
    kinetic = 0.5 * m * np.sum(st["v"] * st["v"], axis=1)
    internal = 0.5 * m * c ** 2 * (st["rho"] - st["rho_ref"]) ** 2 / rho0 ** 2
    return float(np.sum(kinetic + internal))


def initialise(create_cell_list, apply, apply_unary):
    """main() before the time loop (test_collision_2d.jl:123-127); rho0, rho
    and a start at zero as the Particle constructor leaves them."""
    create_cell_list()
    apply(oracle.OP_DENSITY_REF, True)   # find_rho0!, self = true
    apply(oracle.OP_DENSITY, True)       # find_rho!, self = true
    apply_unary(oracle.OP_EOS)           # find_pressure!
    apply(oracle.OP_FORCE, False)        # internal_force!


def run_collision(step, state, count, params, t_end=1.0, on_record=None):
    """The time loop (test_collision_2d.jl:131-140): `step(k)` advances k
    verlet steps.  Returns the recorded particle counts and energies."""
    total, every = collision_schedule(params, t_end)
    N, E = [], []
    done = 0
    for k in range(0, total, every):
        step(k + 1 - done)
        done = k + 1
        st = state()
        N.append(count())
        E.append(energy(st, params))
        if on_record is not None:
            on_record(k, st)
    if total > done:
        step(total - done)
    return np.array(N), np.array(E)


def test_collision_2d_as_written_on_the_oracle(oracle_mod):
    c = G.collision_2d()
    assert c.params["eos"] == 1
    o = oracle_mod.from_case(c)
    initialise(o.create_cell_list, o.apply, o.apply_unary)
    total, every = collision_schedule(c.params)
    assert (total, every) == (4168, 417)
    N, E = run_collision(o.step, o.state, lambda: o.n, c.params)
    assert len(N) == 10
    assert np.all(N == N[0])                     # @testset "count particles"
    assert np.max(E / E[0] - 1.0) < 1e-2         # @testset "energy conservation"
