"""The FP64 drop-in on the benchmark's own system -- the 3D dam break at
dr = 0.0079: 4,096,766 fluid + 1,649,867 wall particles, H = 4 dr -- against
the oracle: cell keys after create_cell_list!, pair-interaction counts per
pass, and every field after the initial state and after each of two
verlet steps, all exactly equal (the FP64 path's bar is 1e-12 relative per
step; it is bit-exact).  The oracle needs ~10 s per step on 16 host cores;
the device holds the system's whole arena (tens of GB)."""
import numpy as np
import pytest

import sphgpu
from sphgpu import geometry as G
from test_gpu_parity import assert_same_state, make

pytestmark = pytest.mark.gpu


def test_dam_break_3d_dr0079_init_and_two_steps_bitexact(gpu, oracle_mod):
    c = G.dam_break(3, 0.0079)
    assert (c.n, c.n_fluid) == (5746633, 4096766)
    g, o = make(c, oracle_mod)
    g.create_cell_list()
    o.create_cell_list()
    assert np.array_equal(g.get("key"), o.keys())
    g.init_state()
    assert g.pair_count(reset=True) == o.init_state()
    assert_same_state(g, o)
    for _ in range(2):
        g.step(1)
        assert g.pair_count(reset=True) == o.step(1)
        assert_same_state(g, o)
    g.synchronize()
    g.close()
