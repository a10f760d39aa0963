"""ParaView export (save_frame!): the frames written asynchronously hold the
fields as they were when save_frame was called, in reference particle order."""
import os

import numpy as np
import pytest

import sphgpu
from sphgpu import geometry as G
from sphgpu.vtk import VtkSeries, read_pvd, read_vtp

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dim,dr", [(2, 0.03), (3, 0.06)])
def test_frames_match_fields(gpu, tmp_path, dim, dr):
    c = G.dam_break(dim, dr)
    g = sphgpu.ParticleSystem(c.params, sphgpu.MIXED)
    g.upload(c.x, c.v, type=c.type)
    g.init_state()
    out = str(tmp_path / "run")
    expect = []
    with VtkSeries(g, out) as series:
        for k in range(4):
            # frames are queued back to back: more than the two buffers in flight
            series.save_frame("v", "rho", "P", "type", time=0.5 * k)
            expect.append({f: g.get(f) for f in ("x", "v", "rho", "P", "type")})
            g.step(3)
    frames = read_pvd(os.path.join(out, "result.pvd"))
    assert [t for t, _ in frames] == [0.0, 0.5, 1.0, 1.5]
    for (t, path), e in zip(frames, expect):
        d = read_vtp(path)
        assert d["n"] == c.n
        assert np.array_equal(d["points"], e["x"])
        assert np.array_equal(d["connectivity"], np.arange(c.n))
        assert np.array_equal(d["offsets"], np.arange(1, c.n + 1))
        pd = d["point_data"]
        assert np.array_equal(pd["v"], e["v"])
        assert np.array_equal(pd["rho"], e["rho"])
        assert np.array_equal(pd["P"], e["P"])
        assert np.array_equal(pd["type"], e["type"])
        assert "x" not in pd


def test_unknown_field_bits_rejected(gpu, tmp_path):
    from sphgpu import _lib as L
    c = G.dam_break(2, 0.05)
    g = sphgpu.ParticleSystem(c.params, sphgpu.FP64)
    g.upload(c.x, c.v, type=c.type)
    s = VtkSeries(g, str(tmp_path / "bad"))
    assert s._lib.sph_vtk_save_frame(s._h, 1 << 20, 0.0, None) == L.SPH_ERR_ARG
    s.save_frame("rho")        # still usable
    s.close()
    assert len(read_pvd(str(tmp_path / "bad" / "result.pvd"))) == 1
