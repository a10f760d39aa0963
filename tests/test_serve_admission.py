"""The served request loop's host logic on the CPU (sphgpu/serve.py), with the
device side replaced by fakes that model each system's device work as a
fixed time per step.  Checked: the HBM budget is never exceeded (charges
include the generator's scratch and the headroom); requests of equal size
are admitted in arrival order; a request that arrives while others run is
admitted as soon as memory frees up (continuous batching); skip-ahead
admission lets small requests pass one that does not fit, until that one
has waited the aging bound; mixed-precision requests of one dimension join
and leave one fused pool between chunks and each still takes exactly its
own step count; every request completes with its results; a request larger
than the whole budget is refused."""
import pytest

import sphgpu
from sphgpu import serve

STEP_TIME = 1.0e-3   # fake device seconds per step
BYTES_PER_PARTICLE = 1000
SCRATCH = 5_000      # fake generator scratch per request


class FakeClock:
    """Each call advances the fake time a little (one loop turn)."""

    def __init__(self):
        self.t = 0.0

    def __call__(self):
        self.t += 2.0e-4
        return self.t


class FakeSystem:
    clock = None
    live = 0
    sizes = {}      # particles per request name

    def __init__(self, params, precision, device=0):
        self.params, self.precision = params, precision
        self.busy_until = 0.0
        self.steps = 0
        self.n = 0
        FakeSystem.live += 1

    def generate(self, shapes):
        self.n = FakeSystem.sizes[shapes[0]["name"]]
        return self.n

    def upload(self, x, v=None, type=None):
        self.n = x.shape[0]

    def init_state(self):
        pass

    def pair_count(self, reset=False):
        return 68 * self.steps * self.n

    def idle(self):
        return FakeSystem.clock.t >= self.busy_until

    def get(self, f):
        return ("field", f, self.steps)

    def close(self):
        FakeSystem.live -= 1


class FakeBatch:
    made = []

    def __init__(self, members):
        self.m = list(members)
        FakeBatch.made.append(len(self.m))

    def step(self, k):
        start = max([FakeSystem.clock.t] + [m.busy_until for m in self.m])
        for m in self.m:
            m.busy_until = start + k * STEP_TIME
            m.steps += k

    def idle(self):
        return all(m.idle() for m in self.m)

    def close(self):
        pass


class _Shapes:
    def __init__(self, name):
        self.shapes = [{"name": name}]
        self.params = {}


@pytest.fixture
def fake_device(monkeypatch):
    clock = FakeClock()
    FakeSystem.clock = clock
    FakeSystem.live = 0
    FakeSystem.sizes = {}
    FakeBatch.made = []
    monkeypatch.setattr(sphgpu, "ParticleSystem", FakeSystem)
    monkeypatch.setattr(sphgpu, "Batch", FakeBatch)
    monkeypatch.setattr(sphgpu, "shape_count",
                        lambda dim, shapes, dev=0: FakeSystem.sizes[shapes[0]["name"]])
    monkeypatch.setattr(sphgpu, "memory_estimate",
                        lambda params, n, precision=0: n * BYTES_PER_PARTICLE)
    monkeypatch.setattr(sphgpu, "generate_scratch", lambda dim, shapes: SCRATCH)
    monkeypatch.setattr(sphgpu, "device_memory", lambda dev=0: (10**12, 10**12))
    monkeypatch.setattr(serve.Request, "shapes", lambda self: _Shapes(f"request{self.rid}"))
    return clock


def _requests(arrivals, steps, sizes=None, precision=0, dim=2):
    sizes = sizes or [1000] * len(arrivals)
    out = []
    for i, (t, s, n) in enumerate(zip(arrivals, steps, sizes)):
        FakeSystem.sizes[f"request{i}"] = n
        out.append(serve.Request(i, dim, 0.02, s, precision, t))
    return out


def charge(n):
    return n * BYTES_PER_PARTICLE + SCRATCH + serve.HEADROOM_BYTES


def test_admission_order_budget_and_continuous_batching(fake_device):
    # room for two systems at a time
    budget = 2 * charge(1000)
    srv = serve.Server(budget_bytes=budget, chunk=10)
    reqs = _requests([0.0, 0.0, 0.001, 0.002], [400, 100, 100, 100])
    done = srv.run(reqs, clock=fake_device)
    assert sorted(r.rid for r in done) == [0, 1, 2, 3]
    assert srv.peak_bytes <= budget and srv.peak_slots == 2
    byid = {r.rid: r for r in done}
    # equal sizes: arrival order
    adm = [byid[i].admitted for i in range(4)]
    assert adm == sorted(adm)
    # request 2 starts when request 1 (short) finishes, while request 0 (long)
    # still runs: continuous batching, not a queue of whole groups
    assert byid[2].admitted >= byid[1].done
    assert byid[2].admitted < byid[0].done
    for r in done:
        assert r.bytes == charge(1000)
        assert r.result["rho"] == ("field", "rho", r.steps)
        assert r.pairs == 68 * r.steps * 1000
        assert r.latency > 0.0
    assert FakeSystem.live == 0


def test_skip_ahead_and_aging_bound(fake_device):
    # request 0 holds most of the budget; request 1 (large) does not fit
    # beside it, requests 2 and 3 (small) do: they pass request 1.  Request 4
    # (small) arrives after request 1 has waited the aging bound: it must
    # wait until request 1 is admitted.
    budget = charge(6000) + charge(2000)
    srv = serve.Server(budget_bytes=budget, chunk=10, max_wait_s=0.05)
    reqs = _requests([0.0, 0.001, 0.002, 0.003, 0.2], [200, 50, 20, 20, 20],
                     sizes=[6000, 5000, 1000, 1000, 1000])
    done = srv.run(reqs, clock=fake_device)
    byid = {r.rid: r for r in done}
    assert sorted(byid) == [0, 1, 2, 3, 4]
    assert byid[2].admitted < byid[1].admitted and byid[3].admitted < byid[1].admitted
    assert srv.skipped_ahead >= 2
    assert srv.aged >= 1
    assert byid[4].admitted >= byid[1].admitted
    assert srv.peak_bytes <= budget
    assert FakeSystem.live == 0


def test_slot_limit(fake_device):
    srv = serve.Server(budget_bytes=10**12, max_slots=1, chunk=10)
    done = srv.run(_requests([0.0, 0.0, 0.0], [20, 20, 20]), clock=fake_device)
    assert len(done) == 3 and srv.peak_slots == 1
    byid = {r.rid: r for r in done}
    assert byid[1].admitted >= byid[0].done and byid[2].admitted >= byid[1].done


def test_mixed_requests_join_and_leave_one_pool(fake_device):
    """Mixed requests of one dimension arriving while others run join the
    pool's fused batch between chunks; each leaves when fewer than a chunk
    of its steps remain and finishes alone; every request takes exactly its
    own step count."""
    steps = [40, 31, 57, 10, 25]
    srv = serve.Server(budget_bytes=10**12, chunk=10)
    reqs = _requests([0.0, 0.0, 0.004, 0.006, 0.05], steps, precision=1)
    done = srv.run(reqs, clock=fake_device)
    byid = {r.rid: r for r in done}
    assert sorted(byid) == [0, 1, 2, 3, 4]
    for i, s in enumerate(steps):
        assert byid[i].result["x"] == ("field", "x", s)   # exactly its steps
        assert byid[i].pooled_steps == s - s % 10
    assert srv.pool_peak_members >= 3          # several requests in one fused batch
    assert srv.pool_rebuilds >= 3              # joins and leaves rebuilt it
    assert max(FakeBatch.made) >= 3
    assert FakeSystem.live == 0


def test_request_beyond_budget_refused(fake_device):
    srv = serve.Server(budget_bytes=500_000)
    with pytest.raises(RuntimeError):
        srv.run(_requests([0.0], [10]), clock=fake_device)


def test_odd_chunks_rejected():
    with pytest.raises(ValueError):
        serve.Server(budget_bytes=1, chunk=5)
