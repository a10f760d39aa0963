"""tests/test_collision_2d.jl restated on the oracle: two colliding circles,
constant particle count and relative energy drift below 1e-2
(test_collision_2d.jl:141-147).  The built-in operators replace the test's
linear EOS by the Tait EOS; with no viscosity and no XSPH the scheme is
conservative, with internal energy e(rho) = B (rho^6/(6 rho_r^7) + 1/rho
- 7/(6 rho_r)) so that de/drho = P/rho^2.  The CPU run stops at t = 0.3
(the circles collide at t ~ 0.1); the GPU test runs the full t = 1.0."""
import numpy as np

from sphgpu import geometry as G


def energy(st, p):
    B = p["c0"] ** 2 * p["rho0"] / 7.0
    m = p["mass"]
    rho, rr = st["rho"], st["rho_ref"]
    e = B * (rho ** 6 / (6.0 * rr ** 7) + 1.0 / rho - 7.0 / (6.0 * rr))
    return float(np.sum(m * (0.5 * np.sum(st["v"] ** 2, axis=1) + e)))


def run_collision(sim, t_end, init, step, state, count):
    c = G.collision_2d()
    init(sim)
    p = c.params
    nsteps = int(round(t_end / p["dt"]))
    frame = max(1, int(round(0.1 / p["dt"])))
    N, E = [], []
    k = 0
    while k <= nsteps:
        step(sim, min(frame, nsteps + 1 - k))
        k += frame
        st = state(sim)
        N.append(count(sim))
        E.append(energy(st, p))
    return np.array(N), np.array(E)


def test_collision_energy_oracle(oracle_mod):
    c = G.collision_2d()
    s = oracle_mod.from_case(c)
    N, E = run_collision(s, 0.3, lambda s: s.init_state(), lambda s, k: s.step(k),
                         lambda s: s.state(), lambda s: s.n)
    assert (N == N[0]).all()
    assert np.max(E / E[0] - 1.0) < 1e-2
