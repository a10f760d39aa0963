"""The served request loop's host logic on the CPU (sphgpu/serve.py), with the
device side replaced by fakes: requests are admitted in arrival order while
their exact device bytes fit in the HBM budget left and a slot is free, a
request that arrives while others run is admitted as soon as memory frees up
(continuous batching, not a queue of whole groups), the budget is never
exceeded, every request completes with its results, and a request larger than
the whole budget is refused.  The fakes model each system's device work as a
fixed time per step on its own stream."""
import pytest

import sphgpu
from sphgpu import serve

STEP_TIME = 1.0e-3   # fake device seconds per step
BYTES_PER_PARTICLE = 1000
PARTICLES = 1000     # every fake request's particle count


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

    def __init__(self, params, precision, device=0):
        self.params, self.precision = params, precision
        self.busy_until = 0.0
        self.steps = 0
        FakeSystem.live += 1

    def generate(self, shapes):
        self.n = PARTICLES  # what the fake shape_count reported for these shapes
        return self.n

    def upload(self, x, v=None, type=None):
        self.n = x.shape[0]

    def init_state(self):
        pass

    def pair_count(self, reset=False):
        return 68 * self.steps * getattr(self, "n", 0)

    def stream(self):
        return 0

    def idle(self):
        return FakeSystem.clock.t >= self.busy_until

    def get(self, f):
        return ("field", f, self.steps)

    def close(self):
        FakeSystem.live -= 1


class FakeBatch:
    def __init__(self, members):
        (self.m,) = members

    def step(self, k):
        m = self.m
        m.busy_until = max(m.busy_until, FakeSystem.clock.t) + k * STEP_TIME
        m.steps += k

    def close(self):
        pass


class FakeEvent:
    def __init__(self, *a, **k):
        self.sys = None

    def record(self, stream):
        self.sys = stream

    def query(self):
        return self.sys.idle()


@pytest.fixture
def fake_device(monkeypatch):
    import torch
    clock = FakeClock()
    FakeSystem.clock = clock
    FakeSystem.live = 0
    monkeypatch.setattr(sphgpu, "ParticleSystem", FakeSystem)
    monkeypatch.setattr(sphgpu, "Batch", FakeBatch)
    monkeypatch.setattr(sphgpu, "shape_count", lambda dim, shapes, dev=0: PARTICLES)
    monkeypatch.setattr(sphgpu, "memory_estimate",
                        lambda params, n, precision=0: n * BYTES_PER_PARTICLE)
    # the loop's CUDA events and external streams: the fake system stands in
    monkeypatch.setattr(torch.cuda, "ExternalStream", lambda s, device=0: FakeSystem._current)
    monkeypatch.setattr(torch.cuda, "Event", FakeEvent)
    return clock


@pytest.fixture(autouse=True)
def _current_system(monkeypatch):
    # ExternalStream(g.stream()) is called right after the system is made:
    # hand the newest fake system to it
    orig = FakeSystem.__init__

    def init(self, *a, **k):
        orig(self, *a, **k)
        FakeSystem._current = self
    monkeypatch.setattr(FakeSystem, "__init__", init)


def _requests(arrivals, steps):
    return [serve.Request(i, 2, 0.02, s, 0, t) for i, (t, s) in enumerate(zip(arrivals, steps))]


def test_admission_order_budget_and_continuous_batching(fake_device):
    # room for two systems at a time (1000 particles x 1000 B each)
    srv = serve.Server(budget_bytes=2_000_000, chunk=10, depth=2)
    reqs = _requests([0.0, 0.0, 0.001, 0.002], [400, 100, 100, 100])
    done = srv.run(reqs, clock=fake_device)
    assert sorted(r.rid for r in done) == [0, 1, 2, 3]
    assert srv.peak_bytes <= 2_000_000 and srv.peak_slots == 2
    byid = {r.rid: r for r in done}
    # arrival order
    adm = [byid[i].admitted for i in range(4)]
    assert adm == sorted(adm)
    # request 2 starts when request 1 (short) finishes, while request 0 (long)
    # still runs: continuous batching, not a queue of whole groups
    assert byid[2].admitted >= byid[1].done
    assert byid[2].admitted < byid[0].done
    for r in done:
        assert r.result["rho"] == ("field", "rho", r.steps)
        assert r.pairs == 68 * r.steps * PARTICLES
        assert r.latency > 0.0
    assert FakeSystem.live == 0


def test_slot_limit(fake_device):
    srv = serve.Server(budget_bytes=10**12, max_slots=1, chunk=10, depth=1)
    done = srv.run(_requests([0.0, 0.0, 0.0], [20, 20, 20]), clock=fake_device)
    assert len(done) == 3 and srv.peak_slots == 1
    byid = {r.rid: r for r in done}
    assert byid[1].admitted >= byid[0].done and byid[2].admitted >= byid[1].done


def test_request_beyond_budget_refused(fake_device):
    srv = serve.Server(budget_bytes=500_000)
    with pytest.raises(RuntimeError):
        srv.run(_requests([0.0], [10]), clock=fake_device)


def test_odd_chunks_rejected():
    with pytest.raises(ValueError):
        serve.Server(budget_bytes=1, chunk=5)
