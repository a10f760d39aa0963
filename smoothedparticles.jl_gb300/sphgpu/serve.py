"""Served stream of dam-break solve requests with continuous batching.

A request asks for one WCSPH dam break (2D or 3D, a lattice spacing, a step
count, FP64 or mixed precision).  The server keeps every admitted system's
state resident on the device between steps and steps all admitted systems
together: each holds a CUDA graph of two fused steps (a one-member ``Batch``)
launched on its own stream, so the work of every admitted request overlaps on
the GPU.  Requests are admitted in arrival order while

* the device bytes the system will hold (``memory_estimate``, exact: the
  library's own arena arithmetic) fit in the HBM budget left, and
* a slot is free (``max_slots``),

so a request that arrives while others run starts as soon as memory and a slot
free up, not when the running ones finish as a group.  Particles are generated
on the device (``ParticleSystem.generate``; the exact count for the admission
test comes from ``shape_count``), or, with ``device_lattice=False``, on host
worker threads from arrival on.  A finished request's fields are copied to the
host, its device memory is released and its completion latency (arrival to
results on the host) is recorded.

Members never interact, and each runs the same launches as ``sph_step``
alone, so every result is bit-identical to running the request by itself.
"""
from __future__ import annotations

import concurrent.futures as cf
import math
import time
from dataclasses import dataclass, field

import numpy as np

from . import geometry as G

RESULT_FIELDS = ("x", "v", "rho", "P")


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


class _Active:
    __slots__ = ("req", "sys", "batch", "issued", "events", "torch_stream")

    def __init__(self, req, sys, batch, torch_stream):
        self.req, self.sys, self.batch = req, sys, batch
        self.issued = 0
        self.events = []
        self.torch_stream = torch_stream


class Server:
    """Continuous-batching request loop on one GPU.

    ``budget_bytes``: device bytes the admitted systems may hold together.
    ``chunk``: steps issued per member at a time (even, so that each chunk is
    graph launches only); up to ``depth`` chunks are queued per member.
    """

    def __init__(self, budget_bytes: int, max_slots: int = 64, chunk: int = 10, depth: int = 2,
                 device: int = 0, workers: int = 4, result_fields=RESULT_FIELDS,
                 device_lattice: bool = True):
        if chunk < 2 or chunk % 2:
            raise ValueError("chunk must be even and >= 2")
        self.budget = int(budget_bytes)
        self.max_slots = max_slots
        self.chunk = chunk
        self.depth = depth
        self.device = device
        self.workers = workers
        self.result_fields = tuple(result_fields)
        self.device_lattice = device_lattice
        self.peak_bytes = 0
        self.peak_slots = 0

    def run(self, requests, clock=time.perf_counter) -> list:
        import torch

        import sphgpu
        reqs = sorted(requests, key=lambda r: r.arrival)
        for r in reqs:
            if r.steps < 0:
                raise ValueError("negative step count")
        pool = cf.ThreadPoolExecutor(max_workers=self.workers)
        futures = {}
        waiting = list(reqs)        # arrived or not, in arrival order
        active: list[_Active] = []
        used = 0
        done = []
        dev = self.device
        t0 = clock()
        try:
            while waiting or active:
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
                            futures[r.rid] = pool.submit(r.case)
                # retire finished members: results to the host, memory released
                still = []
                for a in active:
                    if a.issued >= a.req.steps and a.sys.idle():
                        r = a.req
                        r.result = {f: a.sys.get(f) for f in self.result_fields}
                        r.pairs = a.sys.pair_count()
                        r.done = clock() - t0
                        a.batch.close()
                        a.sys.close()
                        used -= r.bytes
                        done.append(r)
                    else:
                        still.append(a)
                active = still
                # admit in arrival order while memory and slots allow
                while waiting and waiting[0].arrival <= now and len(active) < self.max_slots:
                    r = waiting[0]
                    fut = futures.get(r.rid)
                    if fut is None or not fut.done():
                        break
                    case = fut.result()
                    if self.device_lattice:
                        case, n_case = case
                    else:
                        n_case = case.n
                    need = sphgpu.memory_estimate(case.params, n_case, r.precision)
                    if need > self.budget:
                        raise RuntimeError(f"request {r.rid} needs {need} B, more than the "
                                           f"whole budget {self.budget} B")
                    if used + need > self.budget:
                        break
                    waiting.pop(0)
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
                    b = sphgpu.Batch([g])
                    ts = torch.cuda.ExternalStream(g.stream(), device=dev)
                    active.append(_Active(r, g, b, ts))
                self.peak_bytes = max(self.peak_bytes, used)
                self.peak_slots = max(self.peak_slots, len(active))
                # keep up to `depth` chunks queued per member
                issued_any = False
                for a in active:
                    a.events = [e for e in a.events if not e.query()]
                    while a.issued < a.req.steps and len(a.events) < self.depth:
                        k = min(self.chunk, a.req.steps - a.issued)
                        a.batch.step(k)
                        a.issued += k
                        e = torch.cuda.Event()
                        e.record(a.torch_stream)
                        a.events.append(e)
                        issued_any = True
                if not issued_any:
                    time.sleep(2e-4)
        finally:
            for a in active:
                a.batch.close()
                a.sys.close()
            pool.shutdown(wait=False, cancel_futures=True)
        return done


def summarize(done: list, makespan: float) -> dict:
    lat = np.array([r.latency for r in done])
    pairs = sum(r.pairs for r in done)
    psteps = sum(r.n * r.steps for r in done)
    return {
        "requests": len(done),
        "makespan_s": makespan,
        "p50_latency_s": float(np.percentile(lat, 50)) if len(lat) else None,
        "p99_latency_s": float(np.percentile(lat, 99)) if len(lat) else None,
        "pair_interactions_per_s": pairs / makespan if makespan > 0 else None,
        "particle_steps_per_s": psteps / makespan if makespan > 0 else None,
        "requests_per_s": len(done) / makespan if makespan > 0 else None,
    }
