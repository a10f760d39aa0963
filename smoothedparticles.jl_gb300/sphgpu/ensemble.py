"""The batched ensemble of independent 2D dam breaks.

Each member is the 2D WCSPH dam break (fluid column of width 1.0 in a
4.0 x 3.0 box with 3 wall layers, h = 2.4 dr, support 2h) with its own
column height, viscosity and lattice spacing drawn from a seeded generator:

* column height  ~ U[1.0, 2.0]
* alpha          ~ U[0.01, 0.1]
* fluid particle count target ~ U[2k, 60k]; the spacing is
  dr = sqrt(width * height / count) clamped to [0.004, 0.02]

so the members have uneven particle counts and uneven time steps
(dt = 0.1 h / c0, c0 = 10 sqrt(2 g height)).
"""
from __future__ import annotations

import math

import numpy as np

from . import geometry as G


def ensemble_specs(members: int = 256, seed: int = 2024, n_lo: int = 2000, n_hi: int = 60000):
    """(dr, col_height, alpha) of every member, reproducible from the seed."""
    rng = np.random.default_rng(seed)
    height = rng.uniform(1.0, 2.0, members)
    alpha = rng.uniform(0.01, 0.1, members)
    count = rng.uniform(n_lo, n_hi, members)
    out = []
    for j in range(members):
        dr = math.sqrt(1.0 * height[j] / count[j])
        dr = min(max(dr, 0.004), 0.02)
        out.append((float(dr), float(height[j]), float(alpha[j])))
    return out


def ensemble_cases(members: int = 256, seed: int = 2024, **kw):
    return [G.dam_break(2, dr, col_height=hc, alpha=al, name=f"member{j}")
            for j, (dr, hc, al) in enumerate(ensemble_specs(members, seed, **kw))]
