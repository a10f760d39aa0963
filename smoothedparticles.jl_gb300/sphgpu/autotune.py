"""Autotuner of the pair-pass launch shape for batched ensembles.

The knob is the number of warps per block of the pair passes (2, 4 or 8, i.e.
64, 128 or 256 threads; each warp owns up to 32 targets of one cell, so this
sets how many cell chunks share a block's shared memory and scheduling slot).
Results never depend on it, only the speed does.

* Fused batches (mixed-precision members of one dimension: every kernel of
  the step is one launch over all members) have one setting for the whole
  launch; the tuner times the batched graph with each choice.
* Otherwise every member runs its own launches and is tuned by size class
  (powers of two of the particle count).  A small member stepped alone is
  bound by launch latency, so each class's settings are timed where they run:
  inside the batched graph, with every other class held at its current choice
  (one sweep of coordinate descent, classes largest first).
"""
from __future__ import annotations

import math

CHOICES = (2, 4, 8)


def size_class(n: int) -> int:
    return int(math.log2(max(n, 1)))


def _time(batch, steps: int) -> float:
    """Milliseconds per step of `batch` (graph captured outside the timed
    region)."""
    import torch
    batch.step(2)
    batch.synchronize()
    st = torch.cuda.ExternalStream(batch.stream())
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(st)
    batch.step(steps)
    e1.record(st)
    e1.synchronize()
    return e0.elapsed_time(e1) / steps


def tune_batch(systems, steps: int = 4, choices=CHOICES) -> dict:
    """Chooses warps per block by timing the batched graph; steps the systems
    (their states advance).  Returns {"fused": (warps, {warps: ms})} for a
    fused batch, else {size_class: (warps, {warps: ms})} with every system set
    to its class's choice."""
    import sphgpu
    b = sphgpu.Batch(systems)
    try:
        if b.fused:
            times = {}
            for w in choices:
                b.set_tuning(w)
                times[w] = _time(b, steps)
            best = min(times, key=times.get)
            b.set_tuning(best)
            return {"fused": (best, times)}
    finally:
        b.close()
    classes = {}
    for g in systems:
        classes.setdefault(size_class(g.n), []).append(g)
    weight = {c: sum(g.n for g in gs) for c, gs in classes.items()}
    table = {}
    for c in sorted(classes, key=lambda c: -weight[c]):
        times = {}
        for w in choices:
            for g in classes[c]:
                g.set_tuning(w)
            bb = sphgpu.Batch(systems)
            try:
                times[w] = _time(bb, steps)
            finally:
                bb.close()
        best = min(times, key=times.get)
        for g in classes[c]:
            g.set_tuning(best)
        table[c] = (best, times)
    return table


def apply(systems, table: dict, batch=None):
    """Sets the tuning from a table: the fused setting on `batch`, else every
    system's from the table of its size class."""
    if "fused" in table:
        if batch is not None:
            batch.set_tuning(table["fused"][0])
        return
    for g in systems:
        entry = table.get(size_class(g.n))
        if entry is not None:
            g.set_tuning(entry[0])
