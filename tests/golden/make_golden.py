"""Writes dam_break_oracle.json: SHA-256 digests of the CPU oracle's fields for
small dam breaks, so that the oracle itself is pinned across machines and
compilers and the GPU path is checked against committed values as well as
against the oracle run live.

The reference (SmoothedParticles.jl, Julia) cannot run on these machines, so
these fixtures are the oracle's own outputs: the oracle's pin to the
reference is its restatement of the reference's known-answer tests
(tests/test_kernels.jl, tests/test_collision_2d.jl) and lattice counts.

Each digest covers one field in the reference's particle order, as the raw
little-endian bytes of the float64 (int64 for keys and pairs) array.

    python tests/golden/make_golden.py    # rewrites the JSON beside this file
"""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for _p in (ROOT, os.path.join(ROOT, "smoothedparticles.jl_gb300"), os.path.join(ROOT, "oracle")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

FIELDS = ("x", "v", "a", "xsph", "rho", "rho_ref", "P")
# (dimension, dr, checkpoints in steps after init_state): the 2D case is the
# reference-sized CPU case (5,151 fluid + 1,361 wall particles) over its full
# 200 steps; the 3D case is a small block of the 3D dam break
CASES = [(2, 0.02, (0, 1, 10, 200)), (3, 0.05, (0, 1, 5))]
OUT = os.path.join(HERE, "dam_break_oracle.json")


def digest(a: np.ndarray) -> str:
    a = np.ascontiguousarray(a)
    if a.dtype.kind == "f":
        a = a.astype("<f8", copy=False)
    else:
        a = a.astype("<i8", copy=False)
    return hashlib.sha256(a.tobytes()).hexdigest()


def state_digests(st: dict) -> dict:
    return {f: digest(st[f]) for f in FIELDS}


def run_case(oracle, dim: int, dr: float, checkpoints) -> dict:
    from sphgpu import geometry as G
    case = G.dam_break(dim, dr)
    o = oracle.from_case(case)
    o.create_cell_list()
    rec = {"dim": dim, "dr": dr, "n": int(o.n), "n_fluid": int(case.n_fluid),
           "keys": digest(o.keys()), "pairs": digest(o.pairs()), "n_pairs": int(o.pairs().shape[0])}
    snaps = []
    pairs = o.init_state()
    done = 0
    for c in checkpoints:
        if c > done:
            pairs = 0
            for _ in range(c - done):
                pairs += o.step(1)
            done = c
        st = o.state()
        snaps.append({"steps": c, "pair_interactions": int(pairs),
                      "rho_sum": float(np.sum(st["rho"])), "fields": state_digests(st)})
    rec["snapshots"] = snaps
    o.close()
    return rec


def main() -> None:
    import oracle
    oracle.build()
    oracle.load()
    data = {"note": "SHA-256 of the oracle's fields (reference particle order, little-endian "
                    "float64); pair_interactions = pairs acted on since the previous snapshot "
                    "(init_state's passes for steps 0)",
            "cases": [run_case(oracle, d, dr, cp) for d, dr, cp in CASES]}
    with open(OUT, "w") as f:
        json.dump(data, f, indent=1)
        f.write("\n")
    print(f"wrote {OUT}")


if __name__ == "__main__":
    main()
