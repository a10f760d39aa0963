"""Host-side checks of the ensemble generator and the autotuner's size classes."""
import math

from sphgpu.ensemble import ensemble_specs
from sphgpu import autotune


def test_specs_reproducible_and_in_range():
    a = ensemble_specs(256, seed=11)
    b = ensemble_specs(256, seed=11)
    assert a == b
    assert len(a) == 256
    for dr, hc, al in a:
        assert 0.004 <= dr <= 0.02
        assert 1.0 <= hc <= 2.0
        assert 0.01 <= al <= 0.1
    counts = [hc / (dr * dr) for dr, hc, al in a]
    assert min(counts) < 5000 and max(counts) > 40000
    from sphgpu.ensemble import count_quantiles
    q = count_quantiles(counts)
    assert q["min"] <= q["p25"] <= q["p50"] <= q["p75"] <= q["max"]


def test_size_classes():
    assert autotune.size_class(1) == 0
    assert autotune.size_class(2048) == 11
    assert autotune.size_class(4095) == 11
    assert autotune.size_class(4096) == 12
    assert set(autotune.CHOICES) == {2, 4, 8}


class _FakeSystem:
    def __init__(self, n):
        self.n = n
        self.w = 4

    def set_tuning(self, w):
        self.w = w


def test_apply_table():
    sy = [_FakeSystem(3000), _FakeSystem(50000), _FakeSystem(5000)]
    autotune.apply(sy, {11: (2, {}), 15: (8, {})})
    assert [g.w for g in sy] == [2, 8, 4]
    fused = _FakeSystem(0)           # stands in for a batch
    autotune.apply(sy, {"fused": (8, {})}, fused)
    assert fused.w == 8 and [g.w for g in sy] == [2, 8, 4]


def test_memory_estimate_host_only(sph_lib):
    import sphgpu
    from sphgpu import geometry as G
    c = G.dam_break(2, 0.02)
    a = sphgpu.memory_estimate(c.params, 1000)
    b = sphgpu.memory_estimate(c.params, 2000)
    d = sphgpu.memory_estimate(c.params, 3000)
    assert 0 < a < b < d
    # linear in n up to the 256-byte alignment of each buffer
    assert abs((d - b) - (b - a)) <= 256 * 64
    c3 = G.dam_break(3, 0.05)
    assert sphgpu.memory_estimate(c3.params, 1000) > a  # larger hit lists in 3D
    bad = dict(c.params, h=-1.0)
    try:
        sphgpu.memory_estimate(bad, 10)
    except sphgpu.SphError:
        pass
    else:
        raise AssertionError("negative h accepted")


def test_request_stream_seeded():
    from sphgpu.serve import request_stream, spacing_for, summarize
    a = request_stream(200, rate=2.0, seed=3)
    b = request_stream(200, rate=2.0, seed=3)
    assert [(r.dim, r.dr, r.steps, r.precision, r.arrival) for r in a] == \
           [(r.dim, r.dr, r.steps, r.precision, r.arrival) for r in b]
    arr = [r.arrival for r in a]
    assert arr == sorted(arr) and arr[0] > 0
    assert 60 < arr[-1] < 160  # 200 arrivals at 2/s
    for r in a:
        assert 200 <= r.steps <= 2000 and r.dim in (2, 3) and r.precision in (0, 1)
        n = 2.0 / r.dr ** r.dim
        assert 5e3 * 0.999 <= n <= 2e6 * 1.001
    assert abs(spacing_for(2, 2.0 / 0.01 ** 2) - 0.01) < 1e-15
    assert summarize([], 1.0)["requests"] == 0


def test_dam_break_shapes_params_match_host_case():
    from sphgpu import geometry as G
    for dim, dr, kw in ((2, 0.02, {}), (3, 0.05, dict(lid=True)), (2, 0.01, dict(col_height=1.5))):
        host = G.dam_break(dim, dr, **kw)
        dev = G.dam_break_shapes(dim, dr, **kw)
        assert dev.params == host.params
        assert [s["type"] for s in dev.shapes] == [G.FLUID, G.WALL]
        assert dev.shapes[1]["keep_axis"] == (-1 if kw.get("lid") else dim - 1)


def test_cell_factor_parameter_host_only(sph_lib):
    """sph_params.cell_factor (ABI version 2): mixed systems accept 1..2 and
    hold fewer cells with larger ones; FP64 systems keep the reference's."""
    import pytest
    import sphgpu
    from sphgpu import geometry as G
    c = G.dam_break(2, 0.01)
    base = sphgpu.memory_estimate(c.params, 5000, sphgpu.MIXED)
    larger = sphgpu.memory_estimate(dict(c.params, cell_factor=1.5), 5000, sphgpu.MIXED)
    assert larger < base
    assert sphgpu.memory_estimate(dict(c.params, cell_factor=1.0), 5000, sphgpu.MIXED) == base
    for bad, prec in ((1.5, sphgpu.FP64), (0.9, sphgpu.MIXED), (2.1, sphgpu.MIXED)):
        with pytest.raises(sphgpu.SphError):
            sphgpu.memory_estimate(dict(c.params, cell_factor=bad), 5000, prec)


def test_tune_cell_factor_coordinate_descent(monkeypatch):
    """tune_cell_factor on fakes: every class tried at every factor with the
    other classes at their current choice (largest classes first), the
    trial systems built by `make` and all closed again."""
    import sphgpu
    from sphgpu.geometry import Case  # noqa: F401  (the cases need only .n)

    class FakeCase:
        def __init__(self, n):
            self.n = n

    built, closed = [], []

    class FakeSys:
        def __init__(self, case, f):
            self.case, self.f = case, f
            built.append(self)

        def close(self):
            closed.append(self)

    class FakeBatch:
        def __init__(self, systems):
            self.systems = systems

        def close(self):
            pass

    # cost: class 2^10 prefers 1.15, class 2^12 prefers 1.0
    def fake_time(batch, steps):
        t = 1.0
        for g in batch.systems:
            c = autotune.size_class(g.case.n)
            t += abs(g.f - (1.15 if c == 10 else 1.0)) * g.case.n
        return t

    monkeypatch.setattr(sphgpu, "Batch", FakeBatch)
    monkeypatch.setattr(autotune, "_time", fake_time)
    cases = [FakeCase(1500), FakeCase(1100), FakeCase(5000)]
    table = autotune.tune_cell_factor(cases, FakeSys, steps=2)
    assert table[("cell", 10)][0] == 1.15 and table[("cell", 12)][0] == 1.0
    assert set(table[("cell", 10)][1]) == set(autotune.FACTORS)
    assert len(built) == len(closed) == 2 * len(autotune.FACTORS) * len(cases)
    assert autotune.cell_factors(cases, table) == [1.15, 1.15, 1.0]
    d = autotune.describe(table)
    assert d["cell@2^10"]["choice"] == 1.15
