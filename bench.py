"""Benchmark: pair-interactions/s of the WCSPH dam-break step on GB300.

Workload (default): the 3D dam break at dr = 0.0079 -- 4,096,766 fluid +
1,649,867 wall particles (no lid), H = 4 dr, Wendland quintic, Tait EOS,
artificial viscosity, XSPH, wall pressure, kick-drift-kick -- one `step` is
one verlet_step! of the whole system (binning + density + wall pressure +
force + kick).  Inputs are synthetic lattices generated with the reference's
lattice rules; the 2.6 GB device-resident state is larger than L2, so no L2
flush is needed between steps.

Arms:
  default            this library (FP64 drop-in path), one replica per GPU
  --impl reference   the reference algorithm on the host cores (the C
                     restatement; the Julia reference cannot run here)

Prints one JSON line (rank 0).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "smoothedparticles.jl_gb300")
for _p in (ROOT, PKG, os.path.join(ROOT, "oracle")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

METRIC = "pair-interactions/s, 3D WCSPH 4M ptcl"
UNIT = "pair-interactions/s"
L2_BYTES = 129 * 2**20

# Algorithmic flops of the pair passes (add/sub/mul/compare = 1, a fused
# multiply-add = 2, sqrt = 1, division or reciprocal = 1).  The FP64 path
# evaluates every unordered pair ONCE for both of its targets (sph_tile64.cu)
# and then accumulates each target's row, so its count is per unordered pair
# (the shared work) plus per directed hit (each target's accumulation); the
# mixed path evaluates every directed hit in full (sph_pair32.cu; its density
# pass also the candidates of the live pairs beyond the support, whose shapes
# are zero: not counted), so its count is per directed hit.  3D (2D drops the
# z terms):
#   FP64 density, per unordered pair (fluid-fluid and fluid-wall):
#       d 3 + squares 5 + sqrt 1 + t = 1 - r/H 2 + clamp 1 + m W 6       = 18
#     per directed entry of a fluid target: the row sum 1
#   FP64 wall pressure, per wall entry: W from the stored t 6 + d 3
#       + g.d 5 + the three sums 6                                        = 20
#   FP64 force, per unordered fluid-fluid pair: m rDW 3 + P-sum 1
#       + rho-sum 1 + dv 3 + d 3 + v.d 5 + 2/rho-sum 1 + compare 1
#       + coefficient 2 + m W/rho-bar 1                                   = 21
#     + viscosity where active: r^2 + eta^2 2, reciprocal 1, 3 products  = 6
#     per unordered fluid-wall pair: m rDW 3 + P-sum 1 + coefficient 1
#       + d 3                                                             = 8
#     per directed entry: a += cf d 6 (+ xsph += -wx dv 6, fluid q)
#   mixed, per directed hit: density 18, wall pressure 31, force with a
#     fluid q 55 (wall q 24); the candidate classification is overhead.
FP64_FLOPS = {3: dict(dens_pair=18, dens_entry=1, wall=20, ff_pair=21, av_pair=6, fw_pair=8,
                      acc_a=6, acc_x=6),
              2: dict(dens_pair=15, dens_entry=1, wall=17, ff_pair=17, av_pair=6, fw_pair=7,
                      acc_a=4, acc_x=4)}
MIXED_FLOPS = {3: dict(density=18, wall=31, force_fluid=55, force_wall=24),
               2: dict(density=15, wall=26, force_fluid=45, force_wall=19)}


def pass_flops(cats, dim, mixed):
    """Algorithmic flops of the density, wall-pressure and force passes from
    the hit counts per category (sph_pair_stats: directed hits of the
    operators' targets; the viscosity count is per summed direction)."""
    if mixed:
        F = MIXED_FLOPS[dim]
        return {"density": cats["density"] * F["density"],
                "wall_pressure": cats["wall"] * F["wall"],
                "force": cats["force_fluid"] * F["force_fluid"]
                + cats["force_wall"] * F["force_wall"]}
    F = FP64_FLOPS[dim]
    u_ff = cats["force_fluid"] / 2.0   # both directions of a fluid pair are summed
    u_fw = cats["force_wall"]          # walls are not force targets
    u_av = cats["force_av"] / 2.0
    return {"density": (u_ff + u_fw) * F["dens_pair"] + cats["density"] * F["dens_entry"],
            "wall_pressure": cats["wall"] * F["wall"],
            "force": u_ff * F["ff_pair"] + u_av * F["av_pair"] + u_fw * F["fw_pair"]
            + cats["force_fluid"] * (F["acc_a"] + F["acc_x"]) + cats["force_wall"] * F["acc_a"]}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--dr", type=float, default=0.0079)
    ap.add_argument("--dim", type=int, default=3)
    ap.add_argument("--e2e-steps", type=int, default=0,
                    help="steps of the end-to-end leg (0: the same as --steps)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--error-steps", type=int, default=300,
                    help="steps after which the mixed run is compared with the FP64 run (0: off)")
    # batched ensemble of 2D dam breaks (mixed precision, one CUDA graph)
    ap.add_argument("--ens-members", type=int, default=256)
    ap.add_argument("--ens-steps", type=int, default=1000)
    ap.add_argument("--ens-seed", type=int, default=2024)
    ap.add_argument("--ens-cell-tune", type=int, default=1,
                    help="1: tune the mixed members' cell factor per size class first")
    # served stream of solve requests (continuous batching, HBM budget)
    ap.add_argument("--serve-requests", type=int, default=100)
    ap.add_argument("--serve-rate", type=float, default=2.0, help="arrivals per second")
    ap.add_argument("--serve-min-particles", type=float, default=5e3)
    ap.add_argument("--serve-max-particles", type=float, default=2e6)
    ap.add_argument("--serve-seed", type=int, default=5)
    ap.add_argument("--serve-budget-frac", type=float, default=0.15,
                    help="HBM budget as a fraction of the device memory free at start")
    ap.add_argument("--serve-max-wait", type=float, default=60.0,
                    help="aging bound of the skip-ahead admission (seconds)")
    ap.add_argument("--only", choices=["all", "ensemble", "serve"], default="all")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", str(rank)))
    return rank, world, local


def make_case(args):
    from sphgpu import geometry as G
    return G.dam_break(args.dim, args.dr)


def workload_name(case):
    nf = case.n_fluid
    return (f"{case.dim}D WCSPH dam break dr={case.dr:g}: {nf:,} fluid + {case.n - nf:,} wall "
            f"particles, H={case.params['h']:.5g}, FP64 verlet_step!")


class ClockSampler:
    """nvidia-smi sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.out = ""
        if self.proc:
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                self.out, _ = self.proc.communicate()

    def summary(self):
        rows = []
        for line in (self.out or "").strip().splitlines():
            parts = [t.strip() for t in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(rows)}


def cpu_baseline(case, budget_s=12.0):
    """The oracle (C restatement of the reference's apply! path, OpenMP over
    target particles) on the host cores: density + wall-pressure + force passes
    over a contiguous block of fluid targets of the same system."""
    import oracle
    o = oracle.from_case(case)
    t0 = time.perf_counter()
    o.create_cell_list()
    t_bin = time.perf_counter() - t0
    nf = case.n_fluid
    m = 20000
    lo = nf // 2 - m // 2
    t0 = time.perf_counter()
    o.pair_passes_sample(lo, lo + m)
    t_cal = time.perf_counter() - t0
    m2 = int(min(nf, max(m, m * budget_s / max(t_cal, 1e-3))))
    lo = max(0, nf // 2 - m2 // 2)
    t0 = time.perf_counter()
    pairs = o.pair_passes_sample(lo, lo + m2)
    t = time.perf_counter() - t0
    o.close()
    return dict(value=pairs / t, unit=UNIT, cores=oracle.num_threads(), kind="port",
                sample=(f"pair passes (density, wall pressure, force) over {m2:,} contiguous fluid "
                        f"targets of the same {case.n:,}-particle system: {pairs:,} pairs in "
                        f"{t:.2f} s; create_cell_list! of the full system {t_bin:.2f} s"))


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    import oracle
    case = make_case(args)
    o = oracle.from_case(case)
    o.create_cell_list()
    nf = case.n_fluid
    m = 20000
    lo0 = nf // 2
    t0 = time.perf_counter()
    o.pair_passes_sample(lo0, lo0 + m)
    t_cal = time.perf_counter() - t0
    m = int(min(nf // 4, max(m, m * 6.0 / max(t_cal, 1e-3))))  # ~6 s per step
    pairs_tot, t_tot = 0, 0.0
    for it in range(args.warmup + args.steps):
        lo = (nf // 8 + it * m) % max(1, nf - m)
        t0 = time.perf_counter()
        p = o.pair_passes_sample(lo, lo + m)
        dt = time.perf_counter() - t0
        if it >= args.warmup:
            pairs_tot += p
            t_tot += dt
    value = pairs_tot / t_tot
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * t_tot / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": workload_name(case), "particles": case.n},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": oracle.num_threads(),
                         "kind": "port",
                         "sample": f"each step: density + wall-pressure + force passes over {m:,} "
                                   "contiguous fluid targets (the Julia reference cannot run: no "
                                   "Julia runtime on the box)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def timed_steps(g, torch, dev, steps, world):
    """K steps between CUDA events on the handle's stream (after a barrier),
    with per-kernel event timing and nvidia-smi clock sampling."""
    stream = torch.cuda.ExternalStream(g.stream(), device=dev)
    g.synchronize()
    g.pair_count(reset=True)
    g.pair_stats(reset=True)
    g.reset_kernel_stats()
    g.set_profiling(True)
    l0 = g.launch_count()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize(dev)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(dev) as clk:
        e0.record(stream)
        for _ in range(steps):
            g.step(1)
        e1.record(stream)
        e1.synchronize()
    torch.cuda.synchronize(dev)
    ms = e0.elapsed_time(e1)
    out = dict(ms=ms, launches=g.launch_count() - l0, clocks=clk.summary())
    g.set_profiling(False)
    out["pairs"] = g.pair_count(reset=True)
    out["cats"] = g.pair_stats(reset=True)
    out["kernels"] = {k: v for k, v in g.kernel_stats().items() if v[1] > 0}
    g.synchronize()
    return out


def kernel_table(kst, cats, steps, dim, mixed=False):
    """Per kernel family: total and per-launch time, per-step time and, for the
    pair passes, algorithmic flops per step (the FP64 density and force passes
    of a step are several kernels each: tiles, pair evaluation, row sums)."""
    flops = pass_flops(cats, dim, mixed)
    tot = sum(v[0] for v in kst.values())
    rows = {}
    for k, (tms, nl) in kst.items():
        row = {"ms_total": round(tms, 3), "launches": nl, "ms_avg": round(tms / nl, 4),
               "ms_per_step": round(tms / max(steps, 1), 4),
               "share": round(tms / max(1e-9, tot), 4)}
        if k in flops:
            row["flops_per_step"] = flops[k] / max(steps, 1)
            row["tflops"] = round(flops[k] / (tms * 1e-3) / 1e12, 4)
        rows[k] = row
    return rows


def hbm_peak_gbs():
    """The measured copy bandwidth of the GB300s (driver-written)."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured (MEASURED_PEAKS.json hbm_gbs)"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback 6.8 TB/s"


def binning_roofline(kst, case, mixed: bool):
    """Algorithmic HBM bytes of the step-mode binning kernels over their
    CUDA-event times.  Per particle (d = dimension, fluid moves, walls do not):
      bin_keys    fluid: read x, v, a, xsph (32 d) + type 4, write x, v (16 d)
                  + key 4 + slot 4; wall: read x (8 d) + type 4, write key + slot 8
      bin_scatter read key, slot, rid 12, write 2 indices 8
      bin_rank    read 2 indices 8, write 2 indices 8
      bin_gather  read perm, key, rid 12 + x, v (16 d) + type 4 + rho_ref 8 + oid 8;
                  write x, v (16 d) + rho_ref 8 + type 4 + oid 8 + rid 4 + key 4
                  + cell-relative position 16 + inverse index 4 (+ 16 mixed record)
    Cell tables (scans, item list) are excluded: 4-12 B per cell."""
    d, n, nf = case.dim, case.n, case.n_fluid
    nw = n - nf
    by = {
        "bin_keys": nf * (32 * d + 4 + 16 * d + 8) + nw * (8 * d + 4 + 8),
        "bin_scatter": n * 20,
        "bin_rank": n * 16,
        "bin_gather": n * (12 + 16 * d + 20 + 16 * d + 48 + (16 if mixed else 0)),
    }
    peak, src = hbm_peak_gbs()
    out = {"peak_gbs": peak, "peak_source": src}
    tb, tt = 0, 0.0
    for k, b in by.items():
        if k not in kst:
            continue
        ms = kst[k]["ms_avg"]
        gbs = b / (ms * 1e-3) / 1e9
        out[k] = {"bytes_per_launch": b, "ms_avg": ms, "achieved_gbs": round(gbs, 1),
                  "frac": round(gbs / peak, 3)}
        tb += b
        tt += ms
    if tt > 0:
        all_ms = sum(kst[k]["ms_avg"] * kst[k]["launches"] for k in kst if k.startswith("bin_"))
        steps = max(kst["bin_keys"]["launches"], 1)
        out["particle_kernels"] = {"bytes_per_step": tb, "ms": round(tt, 4),
                                   "achieved_gbs": round(tb / (tt * 1e-3) / 1e9, 1),
                                   "frac": round(tb / (tt * 1e-3) / 1e9 / peak, 3)}
        out["binning_ms_per_step"] = round(all_ms / steps, 4)
    return out


def field_errors(ref, got):
    """Per-field error of `got` against `ref` (dicts of reference-ordered arrays)."""
    out = {}
    for f in ("rho", "P", "a", "xsph", "x", "v"):
        a, b = ref[f], got[f]
        if a.ndim == 2:
            diff = np.linalg.norm(a - b, axis=1)
            scale = np.linalg.norm(a, axis=1)
        else:
            diff = np.abs(a - b)
            scale = np.abs(a)
        out[f] = {"max_abs": float(diff.max()), "rel_norm": float(
            np.linalg.norm(diff) / max(1e-300, np.linalg.norm(scale))),
            "max_rel": float((diff / np.maximum(scale, 1e-300)).max()) if f in ("rho", "x") else None}
    return out


def run_ensemble(args, torch, dev):
    """The batched ensemble: seeded 2D dam breaks of uneven sizes, stepped
    together in mixed precision, two steps per CUDA-graph launch."""
    import sphgpu
    from sphgpu import autotune
    from sphgpu.ensemble import count_quantiles, ensemble_cases
    t0 = time.perf_counter()
    cases = ensemble_cases(args.ens_members, seed=args.ens_seed)
    t_geo = time.perf_counter() - t0

    def make(c, factor):
        g = sphgpu.ParticleSystem(dict(c.params, cell_factor=factor), sphgpu.MIXED, device=dev)
        g.upload(c.x, c.v, type=c.type)
        g.init_state()
        return g

    # the cell size per size class first (the members are rebuilt for each
    # candidate), then the launch shape on the members as built
    t0 = time.perf_counter()
    table = autotune.tune_cell_factor(cases, make, steps=4) if args.ens_cell_tune else {}
    t_cell = time.perf_counter() - t0
    mem = [make(c, f) for c, f in zip(cases, autotune.cell_factors(cases, table))]
    t0 = time.perf_counter()
    table.update(autotune.tune_batch(mem, steps=4))
    t_tune = time.perf_counter() - t0
    b = sphgpu.Batch(mem)
    autotune.apply(mem, table, b)
    b.step(2 * max(2, (args.warmup + 1) // 2))
    b.synchronize()
    for g in mem:
        g.pair_count(reset=True)
    S = max(2, args.ens_steps - args.ens_steps % 2)
    st = torch.cuda.ExternalStream(b.stream(), device=dev)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    l0 = b.stats()["kernels"]
    torch.cuda.synchronize(dev)
    with ClockSampler(dev) as clk:
        e0.record(st)
        b.step(S)
        e1.record(st)
        e1.synchronize()
    ms = e0.elapsed_time(e1)
    pairs = sum(g.pair_count(reset=True) for g in mem)
    bst = b.stats()
    # the same members stepped by sph_step on their own streams (each member
    # replays its own two-step graph: one graph launch per member and step pair)
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    for g in mem:
        g.step(S)
    for g in mem:
        g.synchronize()
    t_plain = time.perf_counter() - t0
    pairs_plain = sum(g.pair_count(reset=True) for g in mem)
    b.close()
    n = [c.n for c in cases]
    for g in mem:
        g.close()
    floor = chain_floor(args, torch, dev, len(cases), bst["kernels_per_graph"] // 2)
    return {
        "workload": (f"{len(cases)} independent 2D dam breaks (seed {args.ens_seed}): dr U[0.004, "
                     "0.02], column height U[1, 2], alpha U[0.01, 0.1]; mixed precision"),
        "particles_total": int(sum(n)), "particles_per_member": count_quantiles(n),
        "steps_timed": S, "ms_per_step": ms / S,
        "value": pairs / (ms * 1e-3), "unit": UNIT,
        "member_steps_per_s": len(cases) * S / (ms * 1e-3),
        "particle_steps_per_s": sum(n) * S / (ms * 1e-3),
        "graph": {"kernels_per_graph": bst["kernels_per_graph"], "steps_per_graph": 2,
                  "graph_launches_timed": S // 2, "kernels_timed": bst["kernels"] - l0,
                  "fused": b.fused,
                  "note": ("fused steps: each kernel of the step is one launch over all members"
                           if b.fused else "one graph branch per member")},
        "unbatched": {"value": pairs_plain / t_plain, "ms_per_step": 1e3 * t_plain / S,
                      "note": "same members, sph_step per member on its own stream (a two-step "
                              "graph of that member alone), host timer"},
        "autotune": autotune.describe(table),
        "tuned": {k: v["choice"] for k, v in autotune.describe(table).items()},
        "autotune_s": t_tune, "cell_tune_s": t_cell, "setup_lattices_s": t_geo,
        "clocks": clk.summary(),
        "l2": "no flush: resident state of all members > 129 MB L2",
        "chain_floor": dict(floor, share_of_step=round(floor["ms_per_step"] / (ms / S), 4)),
    }


def chain_floor(args, torch, dev, members, kernels_per_step, steps=200):
    """The same fused graph (the step's chain of kernels, one launch each over
    all members) on `members` tiny dam breaks (dr = 0.1: ~300 particles each):
    what the chain costs when the kernels have next to nothing to do -- the
    most that fusing the whole step into one persistent launch could save."""
    import sphgpu
    sy = []
    for j in range(members):
        c = __import__("sphgpu.geometry", fromlist=["dam_break"]).dam_break(
            2, 0.1, col_height=1.0 + (j % 5) * 0.2, name=f"tiny{j}")
        g = sphgpu.ParticleSystem(c.params, sphgpu.MIXED, device=dev)
        g.upload(c.x, c.v, type=c.type)
        g.init_state()
        sy.append(g)
    b = sphgpu.Batch(sy)
    b.step(4)
    b.synchronize()
    st = torch.cuda.ExternalStream(b.stream(), device=dev)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(st)
    b.step(steps)
    e1.record(st)
    e1.synchronize()
    ms = e0.elapsed_time(e1) / steps
    kps = b.stats()["kernels_per_graph"] // 2
    parts = sum(g.n for g in sy)
    b.close()
    for g in sy:
        g.close()
    return {"members": members, "particles_total": parts, "ms_per_step": ms,
            "kernels_per_step": kps, "us_per_kernel": round(1e3 * ms / max(kps, 1), 3)}


def run_served(args, torch, dev):
    """A seeded Poisson stream of dam-break solve requests served with
    continuous batching under an HBM budget."""
    import sphgpu
    from sphgpu.serve import Server, request_stream, summarize
    free, total = sphgpu.device_memory(dev)
    budget = int(args.serve_budget_frac * free)
    reqs = request_stream(args.serve_requests, args.serve_rate, seed=args.serve_seed,
                          n_lo=args.serve_min_particles, n_hi=args.serve_max_particles)
    srv = Server(budget, max_slots=64, chunk=10, device=dev, max_wait_s=args.serve_max_wait)
    t0 = time.perf_counter()
    with ClockSampler(dev) as clk:
        done = srv.run(reqs)
    makespan = time.perf_counter() - t0
    out = summarize(done, makespan)
    n = np.array([r.n for r in done])
    out.update({
        "workload": (f"{len(reqs)} requests, Poisson arrivals at {args.serve_rate:g}/s (seed "
                     f"{args.serve_seed}): 2D or 3D dam break, particles log-uniform in "
                     f"[{args.serve_min_particles:g}, {args.serve_max_particles:g}], steps U[200, "
                     "2000], FP64 or mixed"),
        "particles": {"min": int(n.min()), "median": int(np.median(n)), "max": int(n.max())},
        "budget_bytes": budget, "hbm_free_at_start": int(free), "hbm_total_bytes": int(total),
        "peak_admitted_bytes": srv.peak_bytes,
        "peak_admitted_frac": srv.peak_bytes / budget,
        "peak_device_bytes": srv.peak_device_bytes,
        "peak_concurrent": srv.peak_slots,
        "admission": {"skipped_ahead": srv.skipped_ahead, "aging_holds": srv.aged,
                      "max_wait_s": args.serve_max_wait},
        "pools": {"rebuilds": srv.pool_rebuilds, "peak_members": srv.pool_peak_members},
        "latency": "arrival to final fields (x, v, rho, P) on the host",
        "mean_queue_s": float(np.mean([r.admitted - r.arrival for r in done])),
        "clocks": clk.summary(),
    })
    return out


def run_ours(args):
    import torch

    import sphgpu
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = local
    torch.cuda.set_device(dev)
    if args.only != "all":
        leg = run_ensemble(args, torch, dev) if args.only == "ensemble" else run_served(args, torch, dev)
        if rank == 0:
            print(json.dumps({"leg": args.only, **leg}), flush=True)
        return 0
    case = make_case(args)
    fields = ("x", "v", "a", "xsph", "rho", "P")

    # ---- FP64 drop-in: device-resident steps
    g = sphgpu.ParticleSystem(case.params, sphgpu.FP64, device=dev)
    g.upload(case.x, case.v, type=case.type)
    g.init_state()
    for _ in range(args.warmup):
        g.step(1)
    r64 = timed_steps(g, torch, dev, args.steps, world)
    ms_max, pairs_all = r64["ms"], r64["pairs"]
    if world > 1:
        import torch.distributed as dist
        t = torch.tensor([ms_max], device=f"cuda:{dev}")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms_max = float(t.item())
        pt = torch.tensor([float(pairs_all)], device=f"cuda:{dev}", dtype=torch.float64)
        dist.all_reduce(pt)
        pairs_all = float(pt.item())
    value = pairs_all / (ms_max * 1e-3)
    final64 = {f: g.get(f) for f in fields}
    resident = g.memory_usage()

    # ---- end to end through the C ABI with pinned host buffers
    n = g.n
    pin = lambda shape: torch.empty(shape, dtype=torch.float64, pin_memory=True).numpy()
    h = {f: pin((n, 3)) for f in ("x", "v", "a", "xsph")}
    h["rho"], h["P"] = pin((n,)), pin((n,))
    for f in ("x", "v", "a", "xsph"):
        g.get(f, out=h[f])
    g.pair_count(reset=True)
    e2e_steps = args.e2e_steps if args.e2e_steps > 0 else args.steps
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    ins = {f: h[f] for f in ("x", "v", "a", "xsph")}
    outs = {f: h[f] for f in fields}
    for _ in range(e2e_steps):
        g.step_io(ins, outs)
    t_e2e = time.perf_counter() - t0
    e2e = {"value": g.pair_count(reset=True) / t_e2e, "unit": UNIT,
           "h2d_bytes_per_step": int(n * 4 * 24), "d2h_bytes_per_step": int(n * (4 * 24 + 2 * 8)),
           "steps": e2e_steps, "ms_per_step": 1e3 * t_e2e / e2e_steps,
           "note": "per step, one sph_step_io call: x, v, a, xsph set from pinned host arrays, "
                   "one step, x, v, a, xsph, rho, P read into pinned host arrays (reference "
                   "particle order; x after the binning and rho, P after the wall pressure are "
                   "copied while the step's later passes run)"}
    # the FP64 run continues (untimed) to the comparison step
    done64 = args.warmup + args.steps + e2e_steps
    target = max(args.error_steps, done64)
    if args.error_steps > 0 and target > done64:
        g.step(target - done64)
    long64 = {f: g.get(f) for f in fields} if args.error_steps > 0 else None
    g.close()

    # ---- mixed precision: same workload from its own initial state
    gm = sphgpu.ParticleSystem(case.params, sphgpu.MIXED, device=dev)
    gm.upload(case.x, case.v, type=case.type)
    gm.init_state()
    for _ in range(args.warmup):
        gm.step(1)
    rmx = timed_steps(gm, torch, dev, args.steps, world)
    donemx = args.warmup + args.steps
    if args.error_steps > 0:
        gm.step(target - donemx)
    longmx = {f: gm.get(f) for f in fields} if args.error_steps > 0 else None
    mixed = {"value": rmx["pairs"] / (rmx["ms"] * 1e-3), "ms_per_step": rmx["ms"] / args.steps,
             "speedup_vs_fp64": (rmx["pairs"] / rmx["ms"]) / (r64["pairs"] / r64["ms"]),
             "dtype": "fp32 pair arithmetic, fp64 positions/integration/accumulators",
             "error_vs_fp64_after_run": (
                 {"steps": target, "fields": field_errors(long64, longmx),
                  "note": "both runs from their own initial state (init_state of the same lattice)"}
                 if long64 is not None else None),
             "kernels": kernel_table(rmx["kernels"], rmx["cats"], args.steps, case.dim, True),
             "binning_hbm": None,
             "gpu_launches": rmx["launches"], "clocks": rmx["clocks"]}
    # one step from an identical FP64 state (reference density included): the
    # per-step error of the mixed arithmetic
    g = sphgpu.ParticleSystem(case.params, sphgpu.FP64, device=dev)
    g.upload(case.x, case.v, type=case.type)
    g.init_state()
    rho_ref64 = g.get("rho_ref")
    for sysm in (g, gm):
        for f in ("x", "v", "a", "xsph"):
            sysm.set(f, final64[f])
        sysm.set("rho_ref", rho_ref64)
        sysm.step(1)
    one_64 = {f: g.get(f) for f in fields}
    one_mx = {f: gm.get(f) for f in fields}
    g.close()
    gm.close()
    mixed["error_vs_fp64_one_step"] = field_errors(one_64, one_mx)

    # ---- roofline of the dominant kernel of the FP64 step (the force pass)
    kt = kernel_table(r64["kernels"], r64["cats"], args.steps, case.dim)
    mixed["binning_hbm"] = binning_roofline(mixed["kernels"], case, True)
    dom = max((k for k in kt if "tflops" in kt[k]), key=lambda k: kt[k]["ms_total"])
    dfma = sphgpu.pipe_peak("dfma", dev)
    ffma = sphgpu.pipe_peak("ffma", dev)
    peak_tflops = 2.0 * dfma / 1e12
    achieved = kt[dom]["flops_per_step"] / (kt[dom]["ms_per_step"] * 1e-3) / 1e12
    roofline = {"bound": "fp64", "kernel": dom, "achieved": round(achieved, 4),
                "peak": round(peak_tflops, 4), "unit": "TFLOP/s",
                "frac": round(achieved / peak_tflops, 4),
                "per": PASS_KERNELS.get(dom, dom),
                "traffic": NCU_TRAFFIC.get(dom),
                "peak_source": "measured in this run: FP64 FMA issue rate x 2 (sph_pipe_peak); "
                               "MEASURED_PEAKS.json has no FP64 figure",
                "fp32_peak_tflops": round(2.0 * ffma / 1e12, 3),
                "flops_per_pass": kt[dom]["flops_per_step"],
                "ms_per_pass": kt[dom]["ms_per_step"],
                "note": "algorithmic flops of the pair-once algorithm: the shared work of an "
                        "unordered pair once, each target's accumulation once per direction "
                        "(bench.py FP64_FLOPS); sqrt and division count 1 each"}
    # the mixed step's dominant pass against the measured FP32 FMA rate
    kmx = mixed["kernels"]
    mdom = max((k for k in kmx if "tflops" in kmx[k]), key=lambda k: kmx[k]["ms_total"])
    peak32 = 2.0 * ffma / 1e12
    ach32 = kmx[mdom]["flops_per_step"] / (kmx[mdom]["ms_per_step"] * 1e-3) / 1e12
    mixed["roofline"] = {"bound": "fp32", "kernel": mdom, "achieved": round(ach32, 3),
                         "peak": round(peak32, 3), "unit": "TFLOP/s",
                         "frac": round(ach32 / peak32, 4),
                         "note": "per directed hit (the mixed passes evaluate every hit "
                                 "in full; bench.py MIXED_FLOPS)"}

    ensemble = run_ensemble(args, torch, dev) if args.ens_members > 0 else None
    served = run_served(args, torch, dev) if args.serve_requests > 0 else None

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(case)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms_max / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": workload_name(case), "particles": case.n,
                       "fluid": case.n_fluid, "pairs_per_step": r64["pairs"] / args.steps,
                       "l2": l2_note(resident),
                       "replicas": world},
            "steps_per_s": 1e3 * args.steps / ms_max,
            "roofline": roofline, "kernels": kt, "mixed": mixed,
            "binning_hbm": binning_roofline(kt, case, False),
            "ensemble": ensemble, "served": served,
            "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": r64["launches"],
            "clocks": r64["clocks"],
        }
        # a compact digest of the legs, last on the line so that a reader of
        # the output's tail sees it
        line["summary"] = summary(line, resident)
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def _r(v, k=4):
    return None if v is None else float(f"{v:.{k}g}")


def summary(line, resident):
    """The headline figures of every leg in a few hundred bytes."""
    mx, rf = line["mixed"], line["roofline"]
    out = {"fp64": {"ms_per_step": _r(line["ms_per_step"]), "pairs_per_s": _r(line["value"]),
                    "roofline_frac": rf["frac"], "roofline_kernel": rf["kernel"],
                    "e2e_pairs_per_s": _r(line["e2e"]["value"]),
                    "resident_gb": _r(resident / 1e9, 3)},
           "mixed": {"ms_per_step": _r(mx["ms_per_step"]), "pairs_per_s": _r(mx["value"]),
                     "speedup_vs_fp64": _r(mx["speedup_vs_fp64"], 3),
                     "roofline_frac": mx["roofline"]["frac"],
                     "roofline_kernel": mx["roofline"]["kernel"]}}
    one = mx.get("error_vs_fp64_one_step") or {}
    out["mixed"]["err_one_step_rel"] = {f: _r(one[f]["rel_norm"], 2) for f in ("rho", "P", "a", "x")
                                        if f in one}
    run = (mx.get("error_vs_fp64_after_run") or {}).get("fields") or {}
    out["mixed"]["err_after_run_rel"] = {f: _r(run[f]["rel_norm"], 2) for f in ("rho", "P", "a", "x")
                                         if f in run}
    ens = line.get("ensemble")
    if ens:
        out["ensemble"] = {"ms_per_step": _r(ens["ms_per_step"]), "pairs_per_s": _r(ens["value"]),
                           "member_steps_per_s": _r(ens["member_steps_per_s"])}
        if "tuned" in ens:
            out["ensemble"]["tuned"] = ens["tuned"]
    srv = line.get("served")
    if srv:
        out["served"] = {k: _r(srv[k]) if isinstance(srv[k], float) else srv[k]
                         for k in ("requests", "p50_latency_s", "p99_latency_s",
                                   "pair_interactions_per_s", "peak_admitted_frac",
                                   "peak_concurrent") if k in srv}
    cpu = line.get("cpu_baseline")
    if cpu:
        out["cpu_pairs_per_s"] = _r(cpu["value"])
    return out


def l2_note(resident: int) -> str:
    """How the timed steps relate to the 129 MB L2 (no flush between steps)."""
    if resident > L2_BYTES:
        return f"no flush: {resident / 1e9:.1f} GB resident on the device > 129 MB L2"
    return (f"no flush: the {resident / 1e6:.0f} MB resident on the device fit in the 129 MB L2, "
            "so these steps run from L2")


# The kernels of one FP64 force pass of a step (the roofline's unit).
PASS_KERNELS: dict = {"force": "one force pass: frec_build_kernel (particle records) + "
                               "pair_list_kernel (every pair once) + row_sum_kernel (each "
                               "target's row in order) + the overflow sweep of pair64_kernel"}

# DRAM bytes (read + write) of one FP64 force pass from the ncu capture
# summarised in profiles/fp64_tiles_3d_dr0.025.md: frec_build_kernel
# 19,521,024 + 1,280 B, pair_list_kernel 961,587,968 + 1,082,625,024 B and
# row_sum_kernel 1,136,939,520 + 25,849,088 B for the 3D dam break at
# dr = 0.025 (69,489,136 pair-interactions per step), scaled by
# pair-interactions to the 5,746,633-particle case (2,078,775,269 per step).
NCU_TRAFFIC: dict = {"force": int((19521024 + 1280 + 961587968 + 1082625024 + 1136939520
                                   + 25849088) * 2078775269 / 69489136)}


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
