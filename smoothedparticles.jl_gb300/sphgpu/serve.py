"""Served stream of dam-break solve requests with continuous batching.

A request asks for one WCSPH dam break (2D or 3D, a lattice spacing, a step
count, FP64 or mixed precision).  The server keeps every admitted system's
state resident on the device between steps and steps all admitted systems
together, so the work of every admitted request overlaps on the GPU:

* mixed-precision requests of one dimension share a *pool*: one fused batch
  (``Batch`` in fused mode: every kernel of a step is one launch over all
  members, two steps per CUDA-graph launch) that steps its members in chunks
  of ``chunk`` steps.  Between chunks members join (newly admitted requests)
  and leave (a request with fewer than ``chunk`` steps left finishes on its
  own), and the pool's batch is rebuilt -- continuous batching of the
  kernels themselves, not just of streams;
* an FP64 request (and a request finishing its last steps) runs its own
  two-step graph (a one-member ``Batch``) on its own stream.

Admission is by HBM budget.  A request is charged the device bytes its system
will hold (``memory_estimate``), the temporary bytes of the device lattice
generator (``generate_scratch``) and a fixed headroom for the CUDA graphs,
the fused-batch tables and allocation rounding.  Arrived requests are
scanned in arrival order and every one that fits is admitted (skip-ahead:
a request that does not fit does not hold back smaller ones behind it), up
to ``max_slots`` at a time, but a request that has waited ``max_wait_s`` or
longer is not skipped: later ones then wait until it is admitted (the aging
bound that keeps large requests from starving).  A request that arrives
while others run starts as soon as memory and a slot free up.

Progress is polled with the library's own stream queries (``idle``); no
other GPU runtime is needed.  A finished request's fields are copied to the
host, its device memory is released and its completion latency (arrival to
results on the host) is recorded.  Members never interact, and a member of
a fused batch runs the same kernel bodies on the same arguments as
``sph_step`` alone, so every result is bit-identical to running the request
by itself.
"""
from __future__ import annotations

import concurrent.futures as cf
import math
import time
from dataclasses import dataclass, field

import numpy as np

from . import geometry as G

RESULT_FIELDS = ("x", "v", "rho", "P")
HEADROOM_BYTES = 32 * 2**20   # graphs, fused-batch tables, allocation rounding


@dataclass
class Request:
    rid: int
    dim: int
    dr: float
    steps: int
    precision: int
    arrival: float                 # seconds after the stream starts
    col_height: float = 2.0
    alpha: float = 0.02
    # filled by the server
    n: int = 0
    bytes: int = 0
    admitted: float = math.nan
    done: float = math.nan
    pairs: int = 0
    pooled_steps: int = 0          # steps taken as a member of a fused pool
    result: dict = field(default_factory=dict, repr=False)

    @property
    def latency(self) -> float:
        return self.done - self.arrival

    def case(self):
        """The request's particles generated on the host."""
        return G.dam_break(self.dim, self.dr, col_height=self.col_height, alpha=self.alpha,
                           name=f"request{self.rid}")

    def shapes(self):
        """The request's shapes for the device generator (same particles)."""
        return G.dam_break_shapes(self.dim, self.dr, col_height=self.col_height,
                                  alpha=self.alpha, name=f"request{self.rid}")


def spacing_for(dim: int, particles: float) -> float:
    """Lattice spacing whose fluid block (1 x 2 in 2D, 1 x 1 x 2 in 3D)
    holds about `particles` particles."""
    return math.sqrt(2.0 / particles) if dim == 2 else (2.0 / particles) ** (1.0 / 3.0)


def request_stream(count: int, rate: float, seed: int = 5, n_lo: float = 5e3, n_hi: float = 2e6,
                   steps_lo: int = 200, steps_hi: int = 2000, dims=(2, 3), precisions=(0, 1)):
    """Seeded Poisson arrivals (exponential gaps of mean 1/rate seconds).
    Particle counts are log-uniform in [n_lo, n_hi], steps uniform in
    [steps_lo, steps_hi], dimension and precision uniform over the choices."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for i in range(count):
        t += rng.exponential(1.0 / rate)
        dim = int(rng.choice(dims))
        n = math.exp(rng.uniform(math.log(n_lo), math.log(n_hi)))
        steps = int(rng.integers(steps_lo, steps_hi + 1))
        prec = int(rng.choice(precisions))
        out.append(Request(i, dim, spacing_for(dim, n), steps, prec, t))
    return out


class _Member:
    """An admitted request and its device-resident system."""
    __slots__ = ("req", "sys", "issued")

    def __init__(self, req, sys):
        self.req, self.sys = req, sys
        self.issued = 0

    @property
    def left(self) -> int:
        return self.req.steps - self.issued


class _Solo:
    """One system stepping alone (its own two-step graph on its own stream)."""

    def __init__(self, sphgpu, member):
        self.m = member
        self.batch = sphgpu.Batch([member.sys])

    def idle(self) -> bool:
        return self.batch.idle()

    def close(self):
        self.batch.close()


class _Pool:
    """Mixed-precision members of one dimension stepped by one fused batch;
    membership changes between chunks."""

    def __init__(self, dim):
        self.dim = dim
        self.members: list[_Member] = []
        self.joining: list[_Member] = []
        self.batch = None
        self.rebuilds = 0
        self.peak_members = 0

    def idle(self) -> bool:
        return self.batch is None or self.batch.idle()

    def close(self):
        if self.batch is not None:
            self.batch.close()
            self.batch = None


class Server:
    """Continuous-batching request loop on one GPU.

    ``budget_bytes``: device bytes the admitted requests may be charged
    together.  ``chunk``: steps per issue (even, so a pool's chunk is graph
    launches only); a unit gets its next chunk once the previous one has
    finished.  ``max_wait_s``: the aging bound of the skip-ahead admission.
    ``pools``: fuse mixed-precision requests of one dimension (off: every
    request runs alone on its own stream).
    """

    def __init__(self, budget_bytes: int, max_slots: int = 64, chunk: int = 10,
                 device: int = 0, workers: int = 4, result_fields=RESULT_FIELDS,
                 device_lattice: bool = True, max_wait_s: float = 10.0,
                 headroom_bytes: int = HEADROOM_BYTES, pools: bool = True):
        if chunk < 2 or chunk % 2:
            raise ValueError("chunk must be even and >= 2")
        self.budget = int(budget_bytes)
        self.max_slots = max_slots
        self.chunk = chunk
        self.device = device
        self.workers = workers
        self.result_fields = tuple(result_fields)
        self.device_lattice = device_lattice
        self.max_wait_s = max_wait_s
        self.headroom = int(headroom_bytes)
        self.use_pools = pools
        self.peak_bytes = 0
        self.peak_slots = 0
        self.peak_device_bytes = 0
        self.skipped_ahead = 0       # admissions past an earlier request that did not fit
        self.aged = 0                # requests whose wait reached the aging bound (held the rest)
        self._aged_ids = set()
        self.pool_rebuilds = 0
        self.pool_peak_members = 0

    # -- charge of one request
    def _charge(self, sphgpu, r, case, n_case):
        need = sphgpu.memory_estimate(case.params, n_case, r.precision) + self.headroom
        if self.device_lattice:
            need += sphgpu.generate_scratch(r.dim, case.shapes)
        return need

    def run(self, requests, clock=time.perf_counter) -> list:
        import sphgpu
        reqs = sorted(requests, key=lambda r: r.arrival)
        for r in reqs:
            if r.steps < 0:
                raise ValueError("negative step count")
        pool_exec = cf.ThreadPoolExecutor(max_workers=self.workers)
        futures = {}
        waiting = list(reqs)        # not yet admitted, in arrival order
        solos: list[_Solo] = []
        pools = {d: _Pool(d) for d in (2, 3)}
        used = 0
        live = 0
        done = []
        dev = self.device
        free0 = sphgpu.device_memory(dev)[0]
        t0 = clock()

        def retire(m: _Member):
            nonlocal used, live
            r = m.req
            r.result = {f: m.sys.get(f) for f in self.result_fields}
            r.pairs = m.sys.pair_count()
            r.done = clock() - t0
            m.sys.close()
            used -= r.bytes
            live -= 1
            done.append(r)

        try:
            while waiting or solos or live:
                now = clock() - t0
                # arrived requests: shapes and exact particle counts (device
                # generator) or whole lattices on host threads
                for r in waiting:
                    if r.arrival > now:
                        break
                    if r.rid not in futures:
                        if self.device_lattice:
                            sh = r.shapes()
                            fut = cf.Future()
                            fut.set_result((sh, sphgpu.shape_count(r.dim, sh.shapes, dev)))
                            futures[r.rid] = fut
                        else:
                            futures[r.rid] = pool_exec.submit(r.case)
                issued = False
                # solo units: retire when done, else the next chunk
                still = []
                for u in solos:
                    if not u.idle():
                        still.append(u)
                        continue
                    if u.m.left <= 0:
                        u.close()
                        retire(u.m)
                        continue
                    k = min(self.chunk, u.m.left)
                    u.batch.step(k)
                    u.m.issued += k
                    issued = True
                    still.append(u)
                solos = still
                # pools: between chunks, members leave and join, then a chunk
                for p in pools.values():
                    if not p.idle() or not (p.members or p.joining):
                        continue
                    stay, changed = [], bool(p.joining)
                    for m in p.members:
                        if m.left >= self.chunk:
                            stay.append(m)
                            continue
                        changed = True
                        if m.left <= 0:
                            retire(m)
                        else:
                            solos.append(_Solo(sphgpu, m))  # the last few steps alone
                    stay.extend(p.joining)
                    p.joining = []
                    p.members = stay
                    if changed:
                        p.close()
                        if p.members:
                            p.batch = sphgpu.Batch([m.sys for m in p.members])
                            p.rebuilds += 1
                            self.pool_rebuilds += 1
                    if p.members:
                        p.batch.step(self.chunk)
                        for m in p.members:
                            m.issued += self.chunk
                            m.req.pooled_steps += self.chunk
                        p.peak_members = max(p.peak_members, len(p.members))
                        self.pool_peak_members = max(self.pool_peak_members, len(p.members))
                        issued = True
                # admission: skip-ahead in arrival order with an aging bound
                blocked = False
                i = 0
                while i < len(waiting) and live < self.max_slots:
                    r = waiting[i]
                    if r.arrival > now:
                        break
                    fut = futures.get(r.rid)
                    if fut is None or not fut.done():
                        i += 1
                        continue
                    case = fut.result()
                    if self.device_lattice:
                        case, n_case = case
                    else:
                        n_case = case.n
                    need = self._charge(sphgpu, r, case, n_case)
                    if need > self.budget:
                        raise RuntimeError(f"request {r.rid} needs {need} B, more than the "
                                           f"whole budget {self.budget} B")
                    if used + need > self.budget:
                        if now - r.arrival >= self.max_wait_s:
                            if r.rid not in self._aged_ids:
                                self._aged_ids.add(r.rid)
                                self.aged += 1
                            break          # nothing after it may pass it now
                        blocked = True
                        i += 1
                        continue
                    if blocked:
                        self.skipped_ahead += 1
                    waiting.pop(i)
                    del futures[r.rid]
                    g = sphgpu.ParticleSystem(case.params, r.precision, device=dev)
                    if self.device_lattice:
                        g.generate(case.shapes)
                    else:
                        g.upload(case.x, case.v, type=case.type)
                    g.init_state()
                    g.pair_count(reset=True)
                    r.n, r.bytes = n_case, need
                    r.admitted = clock() - t0
                    used += need
                    live += 1
                    m = _Member(r, g)
                    if self.use_pools and r.precision == sphgpu.MIXED and r.steps >= self.chunk:
                        pools[r.dim].joining.append(m)
                    else:
                        solos.append(_Solo(sphgpu, m))
                self.peak_bytes = max(self.peak_bytes, used)
                self.peak_slots = max(self.peak_slots, live)
                self.peak_device_bytes = max(self.peak_device_bytes,
                                             free0 - sphgpu.device_memory(dev)[0])
                if not issued:
                    time.sleep(2e-4)
        finally:
            for u in solos:
                u.close()
                u.m.sys.close()
            for p in pools.values():
                p.close()
                for m in p.members + p.joining:
                    m.sys.close()
            pool_exec.shutdown(wait=False, cancel_futures=True)
        return done


def summarize(done: list, makespan: float) -> dict:
    lat = np.array([r.latency for r in done])
    pairs = sum(r.pairs for r in done)
    psteps = sum(r.n * r.steps for r in done)
    steps = sum(r.steps for r in done)
    return {
        "requests": len(done),
        "makespan_s": makespan,
        "p50_latency_s": float(np.percentile(lat, 50)) if len(lat) else None,
        "p99_latency_s": float(np.percentile(lat, 99)) if len(lat) else None,
        "max_latency_s": float(lat.max()) if len(lat) else None,
        "pair_interactions_per_s": pairs / makespan if makespan > 0 else None,
        "particle_steps_per_s": psteps / makespan if makespan > 0 else None,
        "requests_per_s": len(done) / makespan if makespan > 0 else None,
        "pooled_step_frac": (sum(r.pooled_steps for r in done) / steps) if steps else None,
    }
