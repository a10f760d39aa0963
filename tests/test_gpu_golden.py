"""The FP64 GPU path against the committed oracle digests (tests/golden/):
cell keys, the ordered neighbour-pair list and every field after
init_state and after each checkpoint (the 2D reference-sized dam break over
its full 200 steps, a small 3D block over 5 steps) are bit-identical to the
oracle's, and the pair-interaction counts agree.  Tolerance: exact equality
(the FP64 path reproduces the oracle's evaluation order)."""
import json

import numpy as np
import pytest

import sphgpu
from golden.make_golden import OUT, digest
from sphgpu import geometry as G

pytestmark = pytest.mark.gpu


def cases():
    with open(OUT) as f:
        return json.load(f)["cases"]


@pytest.mark.parametrize("rec", cases(), ids=lambda r: f"{r['dim']}d-{r['dr']}")
def test_gpu_matches_golden(gpu, rec):
    case = G.dam_break(rec["dim"], rec["dr"])
    g = sphgpu.ParticleSystem(case.params, sphgpu.FP64)
    g.upload(case.x, case.v, type=case.type)
    g.create_cell_list()
    assert g.n == rec["n"]
    assert digest(g.get("key")) == rec["keys"]
    pairs = g.debug_pairs()
    assert pairs.shape[0] == rec["n_pairs"]
    assert digest(pairs) == rec["pairs"]
    g.init_state()
    done = 0
    for snap in rec["snapshots"]:
        if snap["steps"] > done:
            g.step(snap["steps"] - done)
            done = snap["steps"]
        assert g.pair_count(reset=True) == snap["pair_interactions"], snap["steps"]
        for f, h in snap["fields"].items():
            assert digest(g.get(f)) == h, f"field {f} after {snap['steps']} steps"
        assert float(np.sum(g.get("rho"))) == snap["rho_sum"]
    g.close()
