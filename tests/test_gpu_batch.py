"""Batched stepping: systems stepped together through one CUDA graph give the
same fields as the same systems stepped alone (exact equality: the graph holds
the very launches of sph_step, only overlapped), for FP64 and mixed precision,
even and odd step counts, after a member is re-uploaded (graph recapture) and
for every warps-per-block setting of the pair passes."""
import numpy as np
import pytest

import sphgpu
from sphgpu import geometry as G
from sphgpu.ensemble import ensemble_cases

pytestmark = pytest.mark.gpu

FIELDS = ("x", "v", "a", "xsph", "rho", "P", "oid")


def make(case, precision):
    g = sphgpu.ParticleSystem(case.params, precision)
    g.upload(case.x, case.v, type=case.type)
    g.init_state()
    return g


def assert_equal(a, b):
    assert a.n == b.n
    for f in FIELDS:
        x, y = a.get(f), b.get(f)
        assert np.array_equal(x, y), f"field {f} differs"


@pytest.mark.parametrize("precision", [sphgpu.FP64, sphgpu.MIXED])
def test_batch_equals_alone(gpu, precision):
    cases = [G.dam_break(2, dr, col_height=hc, alpha=al)
             for dr, hc, al in ((0.04, 2.0, 0.02), (0.05, 1.3, 0.07), (0.03, 1.7, 0.05))]
    mem = [make(c, precision) for c in cases]
    ref = [make(c, precision) for c in cases]
    b = sphgpu.Batch(mem)
    # an odd count leaves the members on the other ping-pong half than the
    # captured graph's: the next graph launch must capture again
    for nsteps in (4, 3, 4, 1, 6):
        b.step(nsteps)
        for r in ref:
            r.step(nsteps)
        b.synchronize()
        for m, r in zip(mem, ref):
            assert_equal(m, r)
    st = b.stats()
    assert st["graph_launches"] == 2 + 1 + 2 + 0 + 3
    assert st["kernels_per_graph"] > 0
    # members keep their own accounting of pairs: same totals as alone
    for m, r in zip(mem, ref):
        assert m.pair_count() == r.pair_count()
    b.close()


def test_batch_recapture_after_upload(gpu):
    big = G.dam_break(2, 0.025, col_height=1.5)
    # member 1 starts with every other particle of `big` (same parameters)
    cases = [G.dam_break(2, 0.04), G.Case("half", 2, big.dr, big.x[::2].copy(),
                                           big.type[::2].copy(), big.v[::2].copy(), big.params)]
    mem = [make(c, sphgpu.MIXED) for c in cases]
    b = sphgpu.Batch(mem)
    b.step(2)
    # the full particle set needs larger buffers: the captured graph is stale
    # and must be captured again
    mem[1].upload(big.x, big.v, type=big.type)
    mem[1].init_state()
    ref = make(big, sphgpu.MIXED)
    b.step(4)
    ref.step(4)
    b.synchronize()
    assert_equal(mem[1], ref)
    assert b.stats()["graph_launches"] == 3


@pytest.mark.parametrize("precision", [sphgpu.FP64, sphgpu.MIXED])
def test_step_graph_equals_single_steps(gpu, precision):
    """sph_step of four or more steps replays a captured graph of the system;
    its fields equal those of the same steps taken one call at a time, for
    even and odd counts in any order (an odd count moves the system to the
    other ping-pong half) and after the system is re-uploaded."""
    c = G.dam_break(2, 0.03)
    g, r = make(c, precision), make(c, precision)
    for nsteps in (6, 5, 4, 5, 5, 1, 7):
        g.step(nsteps)
        for _ in range(nsteps):
            r.step(1)
        assert_equal(g, r)
    assert g.pair_count() == r.pair_count()
    c2 = G.dam_break(2, 0.035)
    for s_ in (g, r):
        s_.upload(c2.x, c2.v, type=c2.type)
        s_.init_state()
    g.step(8)
    for _ in range(8):
        r.step(1)
    assert_equal(g, r)
    if precision == sphgpu.FP64:
        assert g.launch_count() == r.launch_count()


@pytest.mark.parametrize("precision", [sphgpu.FP64, sphgpu.MIXED])
def test_batch_recapture_after_upload_within_capacity(gpu, precision):
    """A member re-uploaded with more particles than when the batch captured
    its steps, but within the buffers it already holds: the captured graph's
    launch sizes are stale, so the batch captures again."""
    big = G.dam_break(2, 0.025, col_height=1.5)
    half = G.Case("half", 2, big.dr, big.x[::2].copy(), big.type[::2].copy(),
                  big.v[::2].copy(), big.params)
    m = make(big, precision)          # buffers for the full set
    m.upload(half.x, half.v, type=half.type)
    m.init_state()
    b = sphgpu.Batch([m])
    b.step(2)                         # captured with the half set's count
    m.upload(big.x, big.v, type=big.type)
    m.init_state()
    ref = make(big, precision)
    b.step(4)
    ref.step(4)
    b.synchronize()
    assert_equal(m, ref)
    assert b.stats()["graph_launches"] == 3
    b.close()


@pytest.mark.parametrize("precision", [sphgpu.FP64, sphgpu.MIXED])
def test_tuning_does_not_change_results(gpu, precision):
    c = G.dam_break(2, 0.03)
    runs = []
    for w in (2, 4, 8):
        g = make(c, precision)
        g.set_tuning(w)
        assert g.tuning() == w
        g.step(5)
        runs.append(g)
    for g in runs[1:]:
        assert_equal(runs[0], g)
    with pytest.raises(sphgpu.SphError):
        runs[0].set_tuning(3)


def test_ensemble_members_batched(gpu):
    """A slice of the seeded ensemble (different sizes, heights, viscosities)."""
    cases = [c for c in ensemble_cases(24, seed=7) if c.n < 15000][:8]
    mem = [make(c, sphgpu.MIXED) for c in cases]
    ref = [make(c, sphgpu.MIXED) for c in cases]
    b = sphgpu.Batch(mem)
    b.step(10)
    for r in ref:
        r.step(10)
    b.synchronize()
    for m, r in zip(mem, ref):
        assert_equal(m, r)


def test_fused_equals_branches_and_alone(gpu):
    """Fused steps (one launch per kernel over all members) against one graph
    branch per member and against stepping alone: identical fields."""
    cases = [c for c in ensemble_cases(24, seed=11) if c.n < 20000][:6]
    fused = [make(c, sphgpu.MIXED) for c in cases]
    branch = [make(c, sphgpu.MIXED) for c in cases]
    ref = [make(c, sphgpu.MIXED) for c in cases]
    bf = sphgpu.Batch(fused)
    bb = sphgpu.Batch(branch)
    bb.set_fused(False)
    for nsteps in (4, 5):
        bf.step(nsteps)
        bb.step(nsteps)
        for r in ref:
            r.step(nsteps)
    bf.synchronize()
    bb.synchronize()
    for a, b2, r in zip(fused, branch, ref):
        assert_equal(a, r)
        assert_equal(b2, r)
        assert a.pair_count() == r.pair_count()
    kf = bf.stats()["kernels_per_graph"]
    kb = bb.stats()["kernels_per_graph"]
    assert kf < 60 < kb            # ~44 launches for two steps of all members
    fp = sphgpu.Batch([make(cases[0], sphgpu.FP64)])
    with pytest.raises(sphgpu.SphError):
        fp.set_fused(True)         # FP64 members step as graph branches


def test_chunk_threads_accuracy_and_batch_identity(gpu):
    """Threads per cell chunk (32/64/128 threads sharing a work item) of the
    mixed passes: the pair set is unchanged (pair counts equal the FP64
    path's), the fields stay within the mixed path's stated bounds of FP64
    (test_gpu_mixed.py), and a fused batch whose members use different
    settings gives each member's fields exactly as stepping it alone."""
    cases = [G.dam_break(2, 0.03), G.dam_break(2, 0.045, col_height=1.4, alpha=0.05),
             G.dam_break(2, 0.025, col_height=1.8)]
    g64 = make(cases[0], sphgpu.FP64)
    g64.step(6)
    for threads in (64, 128):
        g = sphgpu.ParticleSystem(cases[0].params, sphgpu.MIXED)
        g.set_chunk_threads(threads)
        assert g.chunk_threads() == threads
        g.upload(cases[0].x, cases[0].v, type=cases[0].type)
        g.init_state()
        g.step(6)
        assert g.pair_count() == g64.pair_count()
        dx = np.abs(g.get("x") - g64.get("x")).max()
        rho = np.abs(g.get("rho") / g64.get("rho") - 1.0).max()
        assert dx / cases[0].dr <= 1e-6 and rho <= 1e-6, (threads, dx, rho)
        g.close()
    settings = (32, 64, 128)

    def member(c, t):
        g = sphgpu.ParticleSystem(c.params, sphgpu.MIXED)
        g.set_chunk_threads(t)
        g.upload(c.x, c.v, type=c.type)
        g.init_state()
        return g
    mem = [member(c, t) for c, t in zip(cases, settings)]
    ref = [member(c, t) for c, t in zip(cases, settings)]
    b = sphgpu.Batch(mem)
    assert b.fused
    b.set_tuning(2)  # the launch grows to hold the 128-thread member's items
    for nsteps in (4, 3, 6):
        b.step(nsteps)
        for r in ref:
            r.step(nsteps)
        b.synchronize()
        for m, r in zip(mem, ref):
            assert_equal(m, r)
    b.close()
