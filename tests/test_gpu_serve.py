"""The served stream: requests admitted by HBM budget while others run, all
stepped concurrently; each result equals the same request run alone (exact
equality -- members never interact and run the launches of sph_step)."""
import numpy as np
import pytest

import sphgpu
from sphgpu.serve import Request, Server, summarize

pytestmark = pytest.mark.gpu


def alone(r, fields):
    c = r.case()
    g = sphgpu.ParticleSystem(c.params, r.precision)
    g.upload(c.x, c.v, type=c.type)
    g.init_state()
    g.step(r.steps)
    out = {f: g.get(f) for f in fields}
    g.close()
    return out


@pytest.mark.parametrize("device_lattice,pools", [(True, True), (False, True), (True, False)])
def test_served_results_equal_alone(gpu, device_lattice, pools):
    """Requests arriving while others run, admitted by the budget: FP64 ones
    on their own streams, mixed ones of one dimension joining and leaving a
    fused pool between chunks (step counts that are not multiples of the
    chunk, so members leave and finish alone).  Every result equals the same
    request run alone, bit for bit; the budget is never exceeded, neither by
    the charges nor by the device memory actually taken."""
    F, M = sphgpu.FP64, sphgpu.MIXED
    # the 2D mixed requests 2, 5 and 6 arrive together (one pool; they leave
    # at different chunks), request 8 joins them a little later
    reqs = [Request(0, 2, 0.04, 24, F, 0.00), Request(1, 3, 0.08, 10, M, 0.02),
            Request(2, 2, 0.03, 61, M, 0.05), Request(3, 3, 0.06, 12, F, 0.05),
            Request(4, 2, 0.05, 7, F, 0.10, col_height=1.4, alpha=0.06),
            Request(5, 2, 0.035, 42, M, 0.05, col_height=1.1),
            Request(6, 2, 0.045, 26, M, 0.05, col_height=1.7),
            Request(7, 3, 0.09, 18, M, 0.14, alpha=0.05),
            Request(8, 2, 0.04, 30, M, 0.052, col_height=1.3)]
    srv = Server(10**13, max_slots=9, chunk=4, device_lattice=device_lattice, pools=pools)
    charges = []
    for r in reqs:
        c = r.shapes() if device_lattice else r.case()
        n = sphgpu.shape_count(r.dim, c.shapes) if device_lattice else c.n
        charges.append(srv._charge(sphgpu, r, c, n))
    # room for the four largest together: later arrivals may wait for memory
    budget = sum(sorted(charges)[-4:])
    srv.budget = budget
    t = __import__("time").perf_counter()
    done = srv.run(reqs)
    makespan = __import__("time").perf_counter() - t
    assert sorted(r.rid for r in done) == list(range(len(reqs)))
    assert srv.peak_bytes <= budget
    assert srv.peak_device_bytes <= budget
    assert srv.peak_slots <= 9
    if pools:
        assert srv.pool_peak_members >= 2 and srv.pool_rebuilds >= 2
    for r in done:
        assert r.bytes == charges[r.rid]
        assert r.admitted >= r.arrival and r.done >= r.admitted
        ref = alone(r, srv.result_fields)
        for f in srv.result_fields:
            assert np.array_equal(r.result[f], ref[f]), f"request {r.rid}: field {f} differs"
        assert r.pairs > 0
    s = summarize(done, makespan)
    assert s["requests"] == len(reqs) and s["p99_latency_s"] >= s["p50_latency_s"]
    if pools:
        assert s["pooled_step_frac"] > 0


def test_usage_matches_estimate(gpu):
    """Mixed precision: the estimate is the exact allocation.  FP64: the rows
    are sized from the counts of the first density pass; the estimate (a
    full lattice neighbourhood for every particle) bounds them on a dam
    break, and the device's own free memory agrees with the usage."""
    import torch
    r = Request(0, 3, 0.07, 2, sphgpu.MIXED, 0.0)
    c = r.case()
    g = sphgpu.ParticleSystem(c.params, r.precision)
    g.upload(c.x, c.v, type=c.type)
    assert g.memory_usage() == sphgpu.memory_estimate(c.params, c.n, r.precision)
    g.init_state()
    g.step(2)
    assert g.memory_usage() == sphgpu.memory_estimate(c.params, c.n, r.precision)
    g.synchronize()
    assert g.idle()
    g.close()
    r = Request(1, 3, 0.04, 2, sphgpu.FP64, 0.0)
    c = r.case()
    est = sphgpu.memory_estimate(c.params, c.n, r.precision)
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    g = sphgpu.ParticleSystem(c.params, r.precision)
    g.upload(c.x, c.v, type=c.type)
    g.init_state()
    g.step(6)
    g.synchronize()
    used = g.memory_usage()
    assert 0 < used <= est
    # cudaMalloc rounds each allocation up to its page size; the context may
    # reserve local memory for the kernels on their first launch
    taken = free0 - torch.cuda.mem_get_info()[0]
    assert used <= taken <= used + 512 * 2**20
    g.close()
