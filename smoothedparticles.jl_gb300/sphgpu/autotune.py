"""Autotuner of the pair-pass launch shape for batched ensembles.

The knob is the number of warps per block of the pair passes (2, 4 or 8, i.e.
64, 128 or 256 threads; each warp owns up to 32 targets of one cell, so this
sets how many cell chunks share a block's shared memory and scheduling slot).
Results never depend on it, only the speed does.  Members are grouped into
size classes (powers of two of the particle count).  A small member stepped
alone is bound by launch latency, so the tuner times each class's settings
where they run: inside the batched graph, with every other class held at its
current choice (one sweep of coordinate descent, classes largest first).
"""
from __future__ import annotations

import math

CHOICES = (2, 4, 8)


def size_class(n: int) -> int:
    return int(math.log2(max(n, 1)))


def _time_batch(systems, steps: int) -> float:
    """Milliseconds per step of a fresh batch of `systems` (graph captured
    outside the timed region)."""
    import torch

    import sphgpu
    b = sphgpu.Batch(systems)
    try:
        b.step(2)
        b.synchronize()
        st = torch.cuda.ExternalStream(b.stream())
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(st)
        b.step(steps)
        e1.record(st)
        e1.synchronize()
        return e0.elapsed_time(e1) / steps
    finally:
        b.close()


def tune_batch(systems, steps: int = 4, choices=CHOICES) -> dict:
    """Chooses warps per block per size class by timing the whole batch.
    Steps the systems (their states advance); returns
    {size_class: (warps, {warps: ms_per_step})} and leaves every system set
    to its class's choice."""
    classes = {}
    for g in systems:
        classes.setdefault(size_class(g.n), []).append(g)
    current = {c: 4 for c in classes}
    table = {}
    weight = {c: sum(g.n for g in gs) for c, gs in classes.items()}
    for c in sorted(classes, key=lambda c: -weight[c]):
        times = {}
        for w in choices:
            for g in classes[c]:
                g.set_tuning(w)
            times[w] = _time_batch(systems, steps)
        best = min(times, key=times.get)
        current[c] = best
        for g in classes[c]:
            g.set_tuning(best)
        table[c] = (best, times)
    return table


def apply(systems, table: dict):
    """Sets every system's tuning from the table of its size class."""
    for g in systems:
        entry = table.get(size_class(g.n))
        if entry is not None:
            g.set_tuning(entry[0])
