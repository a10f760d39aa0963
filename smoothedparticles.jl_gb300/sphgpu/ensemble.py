"""The batched ensemble of independent 2D dam breaks.

Each member is the 2D WCSPH dam break (fluid column of width 1.0 in a
4.0 x 3.0 box with 3 wall layers, h = 2.4 dr, support 2h) with its own
column height, viscosity and lattice spacing drawn from a seeded generator:

* dr            ~ U[0.004, 0.02]
* column height ~ U[1.0, 2.0]
* alpha         ~ U[0.01, 0.1]

Under the lattice rules these draws give about 2.5k to 125k fluid particles
per member (the realised counts are reported next to every measurement), so
the members have uneven particle counts and uneven time steps
(dt = 0.1 h / c0, c0 = 10 sqrt(2 g height)).
"""
from __future__ import annotations

import numpy as np

from . import geometry as G


def ensemble_specs(members: int = 256, seed: int = 2024):
    """(dr, col_height, alpha) of every member, reproducible from the seed."""
    rng = np.random.default_rng(seed)
    dr = rng.uniform(0.004, 0.02, members)
    height = rng.uniform(1.0, 2.0, members)
    alpha = rng.uniform(0.01, 0.1, members)
    return [(float(dr[j]), float(height[j]), float(alpha[j])) for j in range(members)]


def count_quantiles(counts) -> dict:
    """Realised per-member particle counts: min, quartiles, max."""
    q = np.percentile(np.asarray(counts, dtype=np.float64), [0, 25, 50, 75, 100])
    return {k: int(v) for k, v in zip(("min", "p25", "p50", "p75", "max"), q)}


def ensemble_cases(members: int = 256, seed: int = 2024):
    return [G.dam_break(2, dr, col_height=hc, alpha=al, name=f"member{j}")
            for j, (dr, hc, al) in enumerate(ensemble_specs(members, seed))]
