"""Autotuner of the pair passes' launch shape for batched ensembles.

Three knobs:

* the cell size of mixed-precision members (sph_params.cell_factor: cells of
  1 to 1.3 times the support): larger cells fill more of a warp's 32 lanes
  of targets and of each 32-candidate chunk but add candidates; the pair set never changes, the
  neighbour order (and so the FP32 sums) does.  Chosen per size class on the
  members' initial states (the systems are rebuilt for each candidate);

* warps per block of the pair passes (2, 4 or 8, i.e. 64, 128 or 256
  threads): how many work items (<= 32 targets of one cell each) share a
  block's shared memory and scheduling slot.  Results never depend on it.
* threads per cell chunk of the mixed-precision passes (32, 64 or 128): how
  many warps share one work item, each taking every 1st, 2nd or 4th
  32-candidate chunk of the neighbour sequence.  More threads per item give
  a small member more warps in flight and split long hit lists; the mixed
  results change at the FP32 level (reproducibly per setting).

* Fused batches (mixed-precision members of one dimension: every kernel of
  the step is one launch over all members) have one warps-per-block setting
  for the whole launch, then threads per chunk per size class (powers of two
  of the particle count), each class timed inside the batched graph with
  every other class held at its current choice (one sweep of coordinate
  descent, classes largest first).
* Otherwise every member runs its own launches and is tuned by size class the
  same way (warps per block; threads per chunk for mixed members).
"""
from __future__ import annotations

import math

CHOICES = (2, 4, 8)
THREADS = (32, 64, 128)
FACTORS = (1.0, 1.08, 1.15, 1.22, 1.3)


def size_class(n: int) -> int:
    return int(math.log2(max(n, 1)))


def _time(batch, steps: int) -> float:
    """Milliseconds per step of `batch` (graph captured outside the timed
    region), timed on the batch's stream with the library's own clock-free
    means: host time around a synchronised run of `steps` steps."""
    import time
    batch.step(2)
    batch.synchronize()
    t0 = time.perf_counter()
    batch.step(steps)
    batch.synchronize()
    return 1e3 * (time.perf_counter() - t0) / steps


def _classes(systems):
    classes = {}
    for g in systems:
        classes.setdefault(size_class(g.n), []).append(g)
    weight = {c: sum(g.n for g in gs) for c, gs in classes.items()}
    return classes, sorted(classes, key=lambda c: -weight[c])


def tune_cell_factor(cases, make, steps: int = 4, factors=FACTORS) -> dict:
    """Chooses every size class's cell factor by timing the batched graph of
    all members built by ``make(case, factor)`` (a mixed-precision system at
    its initial state): the class at each candidate, the other classes at
    their current choice (one sweep of coordinate descent, the classes with
    the most particles first).  Returns {("cell", size_class): (factor,
    {factor: ms})}; the trial systems are closed."""
    import sphgpu
    cls = {}
    for c in cases:
        cls.setdefault(size_class(c.n), []).append(c)
    order = sorted(cls, key=lambda k: -sum(c.n for c in cls[k]))
    choice = {k: 1.0 for k in cls}
    table = {}
    for k in order:
        times = {}
        for f in factors:
            trial = dict(choice)
            trial[k] = f
            systems = [make(c, trial[size_class(c.n)]) for c in cases]
            b = sphgpu.Batch(systems)
            try:
                times[f] = _time(b, steps)
            finally:
                b.close()
                for g in systems:
                    g.close()
        choice[k] = min(times, key=times.get)
        table[("cell", k)] = (choice[k], times)
    return table


def cell_factors(cases, table: dict) -> list:
    """Each case's cell factor from a tune_cell_factor table (1 where the
    table has no entry for its size class)."""
    return [table.get(("cell", size_class(c.n)), (1.0, None))[0] for c in cases]


def tune_batch(systems, steps: int = 4, choices=CHOICES, threads=THREADS) -> dict:
    """Chooses the launch shape by timing the batched graph; steps the systems
    (their states advance).  Returns {"fused": (warps, {warps: ms}),
    ("threads", size_class): (threads, {threads: ms}), ...} for a fused batch,
    else {size_class: (warps, {warps: ms}), ("threads", size_class): ...}, with
    every system set to its class's choices."""
    import sphgpu
    classes, order = _classes(systems)
    mixed = {c for c in order if all(g.precision == sphgpu.MIXED for g in classes[c])}
    table = {}
    b = sphgpu.Batch(systems)
    try:
        if b.fused:
            times = {}
            for w in choices:
                b.set_tuning(w)
                times[w] = _time(b, steps)
            best = min(times, key=times.get)
            b.set_tuning(best)
            table["fused"] = (best, times)
            for c in order:
                tt = {}
                for t in threads:
                    for g in classes[c]:
                        g.set_chunk_threads(t)
                    tt[t] = _time(b, steps)
                bt = min(tt, key=tt.get)
                for g in classes[c]:
                    g.set_chunk_threads(bt)
                table[("threads", c)] = (bt, tt)
            return table
    finally:
        b.close()
    for c in order:
        knobs = [("warps", choices)] + ([("threads", threads)] if c in mixed else [])
        for knob, values in knobs:
            times = {}
            for v in values:
                for g in classes[c]:
                    g.set_tuning(v) if knob == "warps" else g.set_chunk_threads(v)
                bb = sphgpu.Batch(systems)
                try:
                    times[v] = _time(bb, steps)
                finally:
                    bb.close()
            best = min(times, key=times.get)
            for g in classes[c]:
                g.set_tuning(best) if knob == "warps" else g.set_chunk_threads(best)
            table[c if knob == "warps" else ("threads", c)] = (best, times)
    return table


def apply(systems, table: dict, batch=None):
    """Sets the tuning from a table: the fused setting on `batch`, every
    system's warps and threads per chunk from the entries of its size class."""
    if "fused" in table and batch is not None:
        batch.set_tuning(table["fused"][0])
    for g in systems:
        c = size_class(g.n)
        entry = table.get(c)
        if entry is not None and "fused" not in table:
            g.set_tuning(entry[0])
        th = table.get(("threads", c))
        if th is not None:
            g.set_chunk_threads(th[0])


def describe(table: dict) -> dict:
    """The table as plain JSON: per size class (particles 2^c .. 2^(c+1)) the
    choices and the timings behind them."""
    out = {}
    for k, (best, times) in table.items():
        key = k if isinstance(k, str) else (f"{'cell' if k[0] == 'cell' else 'threads'}@2^{k[1]}"
                                            if isinstance(k, tuple) else f"warps@2^{k}")
        out[key] = {"choice": best, "ms_per_step": {str(v): round(t, 4) for v, t in times.items()},
                    "spread": round(max(times.values()) / min(times.values()) - 1.0, 4)
                    if min(times.values()) > 0 else 0.0}
    return out
