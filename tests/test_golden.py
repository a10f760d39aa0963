"""The CPU oracle against its committed digests (tests/golden/): the oracle
built on this machine gives, bit for bit, the fields it gave when the
fixtures were written (the 2D reference-sized dam break over its full 200
steps, a small 3D block over 5 steps)."""
import json
import os

import pytest

from golden.make_golden import OUT, run_case


def cases():
    with open(OUT) as f:
        return json.load(f)["cases"]


@pytest.mark.parametrize("rec", cases(), ids=lambda r: f"{r['dim']}d-{r['dr']}")
def test_oracle_matches_golden(oracle_mod, rec):
    got = run_case(oracle_mod, rec["dim"], rec["dr"], [s["steps"] for s in rec["snapshots"]])
    for key in ("n", "n_fluid", "keys", "pairs", "n_pairs"):
        assert got[key] == rec[key], key
    for want, have in zip(rec["snapshots"], got["snapshots"]):
        assert have["pair_interactions"] == want["pair_interactions"], want["steps"]
        for f, h in want["fields"].items():
            assert have["fields"][f] == h, f"field {f} after {want['steps']} steps"


def test_fixture_is_beside_its_generator():
    assert os.path.exists(OUT)
