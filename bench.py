#!/usr/bin/env python3
"""Benchmark of the photon-transport hot path on one GB300.

Workload (default, `--config c1`): the 400-module detector, one isotropic
point emitter inside the hull, 1e8 photons, Frank-Tamm spectrum on 300-800 nm,
Cascadia water, seeds 1..5 (one emitter position per seed; step k uses seed
1 + k % 5).  A "step" is one propagation of all 1e8 photons.

  value  photons/s of the propagation kernel, device-resident inputs, timed with
         CUDA events on the launching stream (L2 flushed between steps by
         writing a 512 MiB buffer).
  e2e    photons/s through the public API call a user makes
         (propagate_photons(setup, hit_buffers)): source upload, kernel,
         counters and the hit rows copied back to host memory, hit table built;
         the context is tuned once beforehand with pp.autotune(setup), outside
         the timed region (skipped with --no-autotune).
  roofline  FP32-issue bound: algorithmic FLOPs of the photon steps taken
         (device counter) / kernel time against a measured FFMA peak.
  cpu_baseline  the CPU oracle (a C restatement of the reference's step
         functions, all host threads) on a bounded sample of the same workload.

`--impl reference` times the reference algorithm on the host cores (the
oracle: the reference itself is Julia/CUDA.jl and is not runnable here).
"""
from __future__ import annotations

import argparse
import json
import os
import re
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
import __graft_entry__ as entry  # noqa: E402

# Algorithmic FP32 operations of one photon step with ONE candidate sphere
# test, counted from the oracle's step body (oracle/pp_oracle_body.inc):
#   step length -log(u)*L .......................... 2 (log counted as 1)
#   ray-sphere test (3 sub, 2 dot3 = 10, b: 3, sqrt 1, d: 1, 2 compares) 20
#   position update 3 FMA ........................... 6
#   path length (+ Kahan 3) and time ................ 6
#   phase function: HG 8, ES 10 + 2 cbrt, mixture 1 .. 21
#   sin(theta) 3, phi 1, sincos 2, new dir 2 ......... 8
#   rotation from e_z (Rodrigues form) ............... 19
FLOPS_PER_STEP = 82

PROFILE_SUMMARY = os.path.join(ROOT, "profiles", "propagate_kernel_c1.txt")


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="c1", choices=["c1", "c0"])
    ap.add_argument("--photons", type=float, default=None)
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--e2e-steps", type=int, default=None)
    ap.add_argument("--no-c2", action="store_true", help="skip the C2 batched-launch report")
    ap.add_argument("--no-c0", action="store_true", help="skip the C0 (README example) report")
    ap.add_argument("--no-proxy", action="store_true",
                    help="skip the reference-algorithm-on-this-GPU report")
    ap.add_argument("--no-surrogate", action="store_true", help="skip the C3/C4 surrogate report")
    ap.add_argument("--c3-pairs", type=float, default=2e6, help="training pairs of the C3 report")
    ap.add_argument("--c3-steps", type=int, default=20000)
    ap.add_argument("--c4-pairs", type=float, default=1e6)
    ap.add_argument("--no-detection", action="store_true", help="skip the PMT detection report")
    ap.add_argument("--detection-records", type=float, default=1e8,
                    help="hit records of the detection report (80 B each, device-resident)")
    ap.add_argument("--surrogate-only", action="store_true",
                    help="print only the C3/C4 surrogate report (for profiling its kernels)")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def workload_name(config: str) -> str:
    """The workload both arms report in `config.workload`."""
    if config == "c1":
        return ("C1: 400 spheres r=0.2159 m on 20 strings (x,y ~ U(-250,250), "
                "z=-250..225 step 25), isotropic point in the hull, 1e8 photons, "
                "Frank-Tamm 300-800 nm, Cascadia water, 15 steps, seeds 1-5")
    return "C0: README single-module example"


def make_setups(pp, config, photons, n_seeds=5):
    if config == "c0":
        out = [pp.workloads.c0_setup(photons, seed=s) for s in range(1, n_seeds + 1)]
    else:
        out = [pp.workloads.c1_setup(photons=photons, seed=s) for s in range(1, n_seeds + 1)]
    # one detector, medium and spectrum shared by all seeds (uploaded once)
    for s in out[1:]:
        s.targets, s.medium, s.spec_dist = out[0].targets, out[0].medium, out[0].spec_dist
        s.spectrum_knots = out[0].spectrum_knots
    return out


def shard_sources(setup, rank, world):
    """Photons of each source split into contiguous ranges, one per rank; the
    Philox streams are keyed on the photon index, so the union of the shards is
    the single-GPU run."""
    import copy
    from importlib import import_module
    pp = import_module(entry.PKG_NAME)
    out = []
    for s in setup.sources:
        n = pp.source_photons(s.photons, setup.photon_scaling)
        lo, hi = n * rank // world, n * (rank + 1) // world
        c = copy.copy(s)
        c.photons = hi - lo
        c.first_photon = lo
        out.append(c)
    return out


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.device = device
        self.samples = []
        self._stop = threading.Event()
        self._proc = None

    def start(self):
        try:
            self._proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, ValueError):
            self._proc = None
            return
        self._t = threading.Thread(target=self._read, daemon=True)
        self._t.start()

    def _read(self):
        for line in self._proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.samples.append(parts)

    def stop(self):
        if self._proc is not None:
            self._proc.terminate()
            try:
                self._proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self._proc.kill()

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in self.samples if s[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for s in self.samples:
            for n, v in zip(names, s[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(self.samples)}


def profile_value(key):
    """A figure of the committed ncu summary of the propagation kernel
    (`key: value` lines), if present."""
    try:
        text = open(PROFILE_SUMMARY).read()
    except OSError:
        return None
    m = re.search(re.escape(key) + r":\s*([0-9.eE+]+)", text)
    return float(m.group(1)) if m else None


def profile_traffic():
    """DRAM bytes per launch from the committed ncu summary, if present."""
    return profile_value("dram_bytes_per_launch_full")


def cpu_baseline(pp, orc, config, seconds, photons_full):
    """The oracle (FP32, all host threads) on a bounded sample of the workload."""
    setup = make_setups(pp, config, photons_full, n_seeds=1)[0]
    nthreads = int(orc.load().ppo_max_threads())
    run = orc.Run.from_setup(setup)
    n_cal = 4000
    t0 = time.perf_counter()
    run.propagate(0, 0, n_cal, nthreads=nthreads, capacity=n_cal)
    dt = time.perf_counter() - t0
    rate0 = n_cal / max(dt, 1e-6)
    # the sample is the first n photons of the seed-1 source
    n = int(min(photons_full, max(n_cal, rate0 * seconds)))
    t0 = time.perf_counter()
    hits, st = run.propagate(0, 0, n, nthreads=nthreads, capacity=n)
    dt = time.perf_counter() - t0
    return {"value": n / dt, "unit": "photons/s", "cores": nthreads, "kind": "port",
            "sample": f"first {n} photons of the seed-1 {config.upper()} source, "
                      f"{len(hits)} hits, {dt:.1f} s"}


def run_reference(args):
    """--impl reference: the reference algorithm (oracle port) on host cores."""
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    pp = entry.load()
    orc = entry.load_oracle()
    orc.build()
    photons = int(args.photons or (1e8 if args.config == "c1" else 1e5))
    nthreads = int(orc.load().ppo_max_threads())
    setups = make_setups(pp, args.config, photons)
    runs = [orc.Run.from_setup(s) for s in setups]
    # size one step's sample to ~1/(steps+warmup) of a ~3 minute budget
    t0 = time.perf_counter()
    runs[0].propagate(0, 0, 2000, nthreads=nthreads, capacity=2000)
    rate = 2000 / max(time.perf_counter() - t0, 1e-6)
    per_step = max(2000, min(photons, int(rate * 150.0 / max(1, args.steps + args.warmup))))
    for k in range(args.warmup):
        runs[k % 5].propagate(0, 0, min(per_step, 2000), nthreads=nthreads, capacity=per_step)
    t0 = time.perf_counter()
    for k in range(args.steps):
        runs[k % 5].propagate(0, 0, per_step, nthreads=nthreads, capacity=per_step)
    dt = time.perf_counter() - t0
    value = per_step * args.steps / dt
    line = {
        "impl": "reference", "metric": "photons/s on 1 GB300", "value": value,
        "unit": "photons/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": dt * 1e3 / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": workload_name(args.config),
                   "implementation": "the reference algorithm on the host cores (CPU oracle port; "
                                     "PhotonPropagation.jl/CUDA.jl is not runnable on this box)",
                   "photons_per_step_sample": per_step, "photons_full": photons},
        "cpu_baseline": {"value": value, "unit": "photons/s", "cores": nthreads, "kind": "port",
                         "sample": f"{per_step} photons per step, {args.steps} steps"},
        "e2e": {"value": value, "unit": "photons/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def bench_c2(pp, torch, local, reps=3):
    """C2: 256 emitters (half isotropic, half cascades; counts log-uniform on
    [1e4, 1e7]) on the C1 detector.  One persistent launch replayed from a CUDA
    graph after autotuning, against 256 sequential plain launches (one per
    source, synchronised after each, as the reference's host loop does)."""
    setup = pp.workloads.c2_setup()
    ctx = pp.Context(local)
    setup.upload(ctx)
    recs = setup.source_records()
    ctx.set_sources(recs, len(setup.sources), 1.0)
    t, _ = ctx.autotune(setup.seed, 15, sample_photons=20_000_000)
    total = ctx.total_photons()
    cap = max(1_000_000, total // 50)
    hits = torch.empty(cap * 80, dtype=torch.uint8, device="cuda")
    ctr = torch.zeros(64, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.Stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    best = 1e30
    for r in range(reps + 1):
        with torch.cuda.stream(stream):
            e0.record(stream)
            ctx.launch(setup.seed, 15, hits.data_ptr(), cap, ctr.data_ptr(), stream.cuda_stream,
                       graph=True)
            e1.record(stream)
        stream.synchronize()
        if r:
            best = min(best, e0.elapsed_time(e1))
    c = ctr.cpu().numpy().view(np.uint64)
    assert int(c[1]) == total and int(c[4]) & 0xffffffff == 0
    batched = total / (best * 1e-3)
    # 256 sequential plain launches
    one = pp._lib.pp_source * 1
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for i in range(len(setup.sources)):
        ctx.set_sources(one(recs[i]), 1, 1.0)
        ctx.launch(setup.seed, 15, hits.data_ptr(), cap, ctr.data_ptr(), stream.cuda_stream)
        stream.synchronize()
    seq_s = time.perf_counter() - t0
    ctx.close()
    return {"workload": "C2: 256 emitters (128 isotropic, 128 cascades a=2.0 b=0.63 "
                        "lrad=0.36 m) uniform in a 1 km cube, counts log-uniform [1e4, 1e7], "
                        "C1 detector", "photons": total,
            "graph_persistent_photons_per_s": batched, "graph_persistent_ms": best,
            "sequential_256_launches_photons_per_s": total / seq_s,
            "sequential_256_launches_ms": seq_s * 1e3,
            "tuning": {"block_threads": t.block_threads, "photons_per_thread": t.photons_per_thread,
                       "cell_size_m": round(float(t.cell_size), 2),
                       "safety_cell_m": round(float(t.safety_cell), 2)}}


def _timed_launches(ctx, torch, seed, photons, reps, cap=2_000_000):
    """Best kernel time (ms) of `reps` launches after one warm-up, device-resident
    inputs and hit buffer, CUDA events on the launching stream; plus the last
    launch's counters."""
    hits = torch.empty(cap * 80, dtype=torch.uint8, device="cuda")
    ctr = torch.zeros(64, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.Stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    best = 1e30
    for r in range(reps + 1):
        with torch.cuda.stream(stream):
            e0.record(stream)
            ctx.launch(seed, 15, hits.data_ptr(), cap, ctr.data_ptr(), stream.cuda_stream)
            e1.record(stream)
        stream.synchronize()
        if r:
            best = min(best, e0.elapsed_time(e1))
    c = ctr.cpu().numpy().view(np.uint64)
    assert int(c[1]) == photons and int(c[4]) & 0xffffffff == 0
    return best, c


def bench_reference_algorithm_gpu(pp, torch, local, ours_photons_per_s, reps=2):
    """A labelled stand-in for the reference's CUDA.jl kernel on this GPU: the
    reference's own algorithm -- every target tested at every step in index
    order (src/photon_prop_cuda.jl:486-506), no culling -- run by this
    library's kernel (tuning target_loop = 1) on the C1 workload (seed 1,
    1e8 photons).  It finds the same hits as the culled kernel; the ratio is
    what the culling and the rest of the design buy on the same hardware.  It
    is not the CUDA.jl kernel itself: Julia is not installed on this machine."""
    setup = pp.workloads.c1_setup(photons=100_000_000, seed=1)
    ctx = pp.Context(local)
    setup.upload(ctx)
    ctx.set_sources(setup.source_records(), len(setup.sources), 1.0)
    ctx.set_tuning(target_loop=1)
    ms, c = _timed_launches(ctx, torch, setup.seed, 100_000_000, reps)
    ctx.close()
    rate = 1e8 / (ms * 1e-3)
    return {"workload": "C1, seed 1, 1e8 photons", "photons_per_s": rate, "ms": ms,
            "hits": int(c[0]),
            "ours_over_proxy": ours_photons_per_s / rate if ours_photons_per_s else None,
            "what": "the reference's brute-force target loop (all 400 spheres tested in index "
                    "order at every step, src/photon_prop_cuda.jl:486-506) run by this "
                    "library's kernel on the same GB300 (tuning target_loop=1): a proxy for the "
                    "reference CUDA.jl kernel, not that kernel (Julia is unavailable on this box)"}


def bench_c0(pp, torch, local, reps=20):
    """C0, the README example (one isotropic point at the origin, 1e5 photons at
    450 nm, one module r = 0.3 m at 10 m, seed 1): photons/s of the kernel and
    through propagate_photons, the module's hit count and the arrival-time
    histogram in 1 ns bins on 0-500 ns.  The histogram of a 1e7-photon run is
    compared with the oracle's on an independent stream (two-sample Poisson
    chi-square; 1e5 photons give ~25 hits, too few for a comparison)."""
    from scipy import stats
    setup = pp.workloads.c0_setup(100_000, seed=1)
    ctx = pp.Context(local)
    setup.upload(ctx)
    ctx.set_sources(setup.source_records(), 1, 1.0)
    ms, c = _timed_launches(ctx, torch, setup.seed, 100_000, reps, cap=100_000)
    ctx.close()
    hb = pp.HitBuffers(100_000, local)
    pp.propagate_photons(setup, hb)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(reps):
        table = pp.propagate_photons(setup, hb)
    e2e_s = (time.perf_counter() - t0) / reps
    edges = np.arange(0.0, 501.0, 1.0)
    hist, _ = np.histogram(table["time"], edges)
    # power: 1e7 photons on both sides, independent streams
    big_g = pp.workloads.c0_setup(10_000_000, seed=60)
    big_o = pp.workloads.c0_setup(10_000_000, seed=61)
    tg = pp.propagate_photons(big_g, pp.HitBuffers(1_000_000, local))
    orc = entry.load_oracle()
    orc.build()
    want, _ = orc.Run.from_setup(big_o).propagate()
    hg, _ = np.histogram(tg["time"], edges)
    ho, _ = np.histogram(want["time"], edges)
    big = (hg + ho) >= 10
    A = np.append(hg[big], hg[~big].sum()).astype(float)
    B = np.append(ho[big], ho[~big].sum()).astype(float)
    keep = (A + B) > 0
    chi2 = float(np.sum((A[keep] - B[keep]) ** 2 / (A[keep] + B[keep])))
    dof = int(keep.sum())
    nz = np.nonzero(hist)[0]
    return {"workload": "C0: README example, 1e5 photons, 450 nm, module r=0.3 m at (0,0,10) m, "
                        "seed 1",
            "kernel_photons_per_s": 1e5 / (ms * 1e-3), "kernel_ms": ms,
            "e2e_photons_per_s": 1e5 / e2e_s, "e2e_ms": e2e_s * 1e3,
            "hits": int(table.nrow), "per_module": {"1": int(table.nrow)},
            "time_hist_1ns_0_500": {"first_bin_ns": 0, "nonzero_bins": nz.tolist(),
                                     "counts": hist[nz].tolist()},
            "vs_oracle_1e7": {"gpu_hits": int(tg.nrow), "oracle_hits": int(len(want)),
                              "hist_chi2": chi2, "dof": dof,
                              "p": float(stats.chi2.sf(chi2, dof)),
                              "count_z": (tg.nrow - len(want)) / np.sqrt(tg.nrow + len(want)),
                              "streams": "GPU seed 60, oracle seed 61"}}


def bench_surrogate(pp, torch, local, args):
    """C3: MC tables (1e5 photons per pair, histogram mode) and Adam training
    of the 8 -> 4x256 SiLU -> 1+64 network at batch 8192, lr 1e-3.
    C4: one batch of 1e6 pairs answered by the fused inference kernel, 1% of
    pairs audited by the MC at 1e7 photons (the judge), errors of the network
    against it on the audited pairs with at least 400 MC hits."""
    s = pp.surrogate
    ctx = pp.Context(local)
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except OSError:
        pass
    table_ph = 100_000
    n3 = int(args.c3_pairs)
    pairs = s.sample_pairs(n3, seed=1)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    c, h = s.generate_tables(pairs, table_ph, seed=1, ctx=ctx, device_out=True)
    t_tab = time.perf_counter() - t0
    x = torch.tensor(s.pair_features(pairs), device="cuda")
    mlp = s.MLP(device=local, max_batch=8192, seed=0)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    log = s.train(mlp, x, c, h, steps=args.c3_steps, batch=8192, lr=1e-3,
                  log_every=max(1, args.c3_steps // 20))
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    # one training step timed alone with events (forward, backward, Adam)
    bi = torch.randint(0, n3, (8192,), device="cuda")
    bx, bc, bh = x[bi].contiguous(), c[bi].contiguous(), h[bi].contiguous()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    cur = torch.cuda.current_stream().cuda_stream
    e0.record()
    for _ in range(20):
        mlp.train_step(bx.data_ptr(), bc.data_ptr(), bh.data_ptr(), 8192, 1e-6, stream=cur)
    e1.record()
    torch.cuda.synchronize()
    step_ms = e0.elapsed_time(e1) / 20
    # the same step as captured replays (batch drawn on the device included)
    xp = [t.data_ptr() for t in (x, c, h)]
    mlp.train_steps(*xp, n3, 8192, 3, 0, 10**9, 1e-6, 1e-6, 5, stream=cur)
    e0.record()
    mlp.train_steps(*xp, n3, 8192, 20, 0, 10**9, 1e-6, 1e-6, 5, stream=cur)
    e1.record()
    torch.cuda.synchronize()
    graph_step_ms = e0.elapsed_time(e1) / 20
    flops_row = 2 * sum(r * cc for r, cc in
                        (mlp.layout(l)[2:] for l in range(mlp.n_layers + 1)))
    # C4
    n4 = int(args.c4_pairs)
    ev = s.sample_pairs(n4, seed=4)
    xb = torch.tensor(s.pair_features(ev), device="cuda")
    eb = torch.empty(n4, device="cuda")
    pb = torch.empty((n4, s.N_BINS), device="cuda")
    for _ in range(3):
        mlp.infer(xb.data_ptr(), n4, eb.data_ptr(), pb.data_ptr(), stream=cur, check_now=False)
    torch.cuda.synchronize()
    e0.record()
    for _ in range(10):
        mlp.infer(xb.data_ptr(), n4, eb.data_ptr(), pb.data_ptr(), stream=cur, check_now=False)
    e1.record()
    torch.cuda.synchronize()
    mlp.infer(xb.data_ptr(), n4, eb.data_ptr(), pb.data_ptr())  # checks the error flag
    infer_ms = e0.elapsed_time(e1) / 10
    # a failed audit is reported (audit.passed) rather than re-run through the MC
    sur = s.Surrogate(mlp, table_photons=table_ph, ctx=ctx, on_failure="flag")
    t0 = time.perf_counter()
    r = sur.expectations(ev, photons=table_ph, seed=5)
    t_batch = time.perf_counter() - t0
    a = r.audit
    mc_rate = a["mc_pairs"] / a["mc_seconds"] if a["mc_seconds"] > 0 else None
    # the methods without the network, on the audited pairs the MC judged
    aud = np.flatnonzero(r.from_mc)
    judge = r.counts[aud] * (1e7 / table_ph)
    ok = judge >= 400
    gain = None
    if ok.sum() >= 5:
        sub = ev.subset(aud[ok])
        lc, _ = s.generate_tables(sub, table_ph, seed=6, ctx=ctx)
        rel_mc = np.abs(lc * (1e7 / table_ph) - judge[ok]) / judge[ok]
        norm = s.fit_analytic_norm(sub, judge[ok], 1e7)
        rel_an = np.abs(s.analytic_expectation(sub, 1e7, norm=norm) - judge[ok]) / judge[ok]
        gain = {"equal_cost_mc_1e5_median_rel_error": float(np.median(rel_mc)),
                "analytic_scaling_median_rel_error": float(np.median(rel_an)),
                "analytic": "norm*N*r^2/(4d^2)*exp(-d/25 m), norm fitted to the judge"}
    mlp.close()
    ctx.close()
    bf16_peak = peaks.get("bf16_tflops")
    infer_tflops = flops_row * n4 / (infer_ms * 1e-3) / 1e12
    return {
        "c3_training": {
            "workload": f"{n3} pairs (d log-uniform [5, 300] m, directions uniform), "
                        f"{table_ph} photons per pair, cascades a=2.0 b=0.63 lrad=0.36 m, "
                        "targets: count + 64-bin log10(t_res+21 ns) histogram",
            "table_photons_per_s": n3 * table_ph / t_tab, "table_seconds": t_tab,
            "train_steps": args.c3_steps, "batch": 8192, "lr": 1e-3,
            "train_seconds": t_train, "train_step_ms": step_ms,
            "train_tflops": 3 * flops_row * 8192 / (step_ms * 1e-3) / 1e12,
            "train_step_graph_ms": graph_step_ms,
            "train_tflops_graph": 3 * flops_row * 8192 / (graph_step_ms * 1e-3) / 1e12,
            "loss_first": log[0][1], "loss_last": log[-1][1]},
        "c4_inference": {
            "workload": f"{n4} pairs from the training distributions; 1% audited by the MC "
                        "at 1e7 photons per pair",
            "nn_module_expectations_per_s": n4 / (infer_ms * 1e-3),
            "infer_ms": infer_ms,
            "roofline": {"bound": "tensor", "achieved": infer_tflops, "peak": bf16_peak,
                         "unit": "TFLOP/s",
                         "frac": infer_tflops / bf16_peak if bf16_peak else None,
                         "note": f"{flops_row} FLOPs per pair; peak = measured cuBLAS bf16"},
            "batch_module_expectations_per_s": n4 / t_batch, "batch_seconds": t_batch,
            "mc_1e7_module_expectations_per_s": mc_rate,
            "speedup_nn_only": (n4 / (infer_ms * 1e-3)) / mc_rate if mc_rate else None,
            "speedup_with_audit": (n4 / t_batch) / mc_rate if mc_rate else None,
            "audit": a, "without_network": gain},
    }


def bench_detection(pp, torch, local, n=100_000_000, reps=5):
    """Photon hits -> PMT hits (pp_make_hits_from_photons) on 1e8 synthetic hit
    records on 400 POMs at the C1 module positions (positions uniform on the
    module surfaces, wavelengths with density 1/lambda^2 on 300-800 nm),
    device-resident;
    8 GB of records, so every launch streams from HBM."""
    import ctypes
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pmt_oracle
    pom = pp.pom
    det, _ = pp.workloads.detector_400()
    targets = [pom.POM.at(t.shape.position, t.module_id) for t in det]
    centres = torch.tensor(np.array([t.shape.position for t in targets], np.float32),
                           device="cuda")
    g = torch.Generator(device="cuda")
    g.manual_seed(1)
    rec = torch.zeros((n, 20), dtype=torch.float32, device="cuda")  # 80-byte records
    mi = torch.randint(0, len(targets), (n,), device="cuda", generator=g)
    v = torch.randn((n, 3), device="cuda", generator=g)
    v /= v.norm(dim=1, keepdim=True)
    rec[:, 0:3] = centres[mi] + pom.POM_RADIUS * v
    del v
    u = torch.rand(n, device="cuda", generator=g)
    rec[:, 3] = 1.0 / (1.0 / 300.0 - u * (1.0 / 300.0 - 1.0 / 800.0))  # density 1/lambda^2
    del u
    rec[:, 7] = (mi + 1).to(torch.int32).view(torch.float32)  # module_index
    ids = torch.empty(n, dtype=torch.int32, device="cuda")
    qe = torch.empty(n, dtype=torch.float32, device="cuda")
    tg = pp.detection.pmt_targets(targets)
    model = pom.pom_model()
    lib = pp._lib.load()
    stream = torch.cuda.current_stream().cuda_stream

    def launch(seed):
        pp._lib.check(lib.pp_make_hits_from_photons(ctypes.c_void_p(rec.data_ptr()), n, tg,
                                                    len(targets), ctypes.byref(model), seed,
                                                    ctypes.c_void_p(ids.data_ptr()),
                                                    ctypes.c_void_p(qe.data_ptr()),
                                                    ctypes.c_void_p(stream)))
    for k in range(3):
        launch(k)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for k in range(reps):
        launch(10 + k)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    detected = int((ids > 0).sum().item())
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except OSError:
        pass
    hbm = peaks.get("hbm_gbs")
    algo = 40.0  # bytes per hit: 2 x 16 B of the record read, 4 B id + 4 B QE written
    achieved = n * algo / (ms * 1e-3) / 1e9
    # CPU: the numpy oracle (one thread) on a bounded sample of the same records
    m = min(n, 2_000_000)
    host = rec[:m].cpu().numpy()
    t = pom.load_pom_tables()
    model_d = dict(acc_wavelength=t.acc_wavelength, acc_group1=t.acc_group1,
                   acc_group2=t.acc_group2, sigma_group1=t.sigma_group1,
                   sigma_group2=t.sigma_group2, qe_wavelength=t.qe_wavelength, qe=t.qe,
                   pmt_dir=pom.pom_pmt_directions(), pmt_group=pom.POM_PMT_GROUP)
    otargets = [dict(position=x.shape.position, radius=x.shape.radius, kind="pom",
                     active_area=x.pmt_area) for x in targets]
    t0 = time.perf_counter()
    pmt_oracle.detect(host[:, 0:3], host[:, 3], host[:, 7].view(np.int32), otargets, model_d, 0)
    cpu_rate = m / (time.perf_counter() - t0)
    del rec, ids, qe, mi
    torch.cuda.empty_cache()
    return {"workload": f"{n:.0e} hit records on 400 POMs (C1 positions), uniform on the module "
                        "surfaces, 1/lambda^2 wavelengths on 300-800 nm; records resident in "
                        f"HBM ({n * 80 / 1e9:.1f} GB)",
            "hits_per_s": n / (ms * 1e-3), "ms": ms, "detected_fraction": detected / n,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                         "frac": achieved / hbm if hbm else None,
                         "note": "40 algorithmic bytes per hit; peak = measured copy bandwidth. "
                                 "The kernel is instruction-issue bound, not HBM-bound: each hit "
                                 "evaluates acos, sqrt and exp2 for 16 PMTs"},
            "cpu_baseline": {"value": cpu_rate, "unit": "hits/s", "cores": 1, "kind": "port",
                             "sample": f"numpy oracle on the first {m} records"}}


def run_ours(args):
    import torch
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    pp = entry.load()
    photons = int(args.photons or (1e8 if args.config == "c1" else 1e5))
    setups = make_setups(pp, args.config, photons)
    ctxs = []
    for s in setups:
        c = pp.Context(local)
        s.upload(c)
        srcs = shard_sources(s, rank, world) if world > 1 else s.sources
        from importlib import import_module
        recs = import_module(entry.PKG_NAME).sources.to_records(srcs)
        c.set_sources(recs, len(srcs), s.photon_scaling)
        c._recs = recs
        ctxs.append(c)
    tuning = None
    if not args.no_autotune:
        t, rate = ctxs[0].autotune(setups[0].seed, 15, sample_photons=min(photons, 8_000_000))
        tuning = dict(block_threads=t.block_threads, photons_per_thread=t.photons_per_thread,
                      cell_size=t.cell_size)
        for c in ctxs[1:]:
            c.set_tuning(**tuning)
    photons_rank = ctxs[0].total_photons()

    cap = max(1_000_000, photons_rank // 20)
    hits = torch.empty(cap * 80, dtype=torch.uint8, device="cuda")
    counters = torch.zeros(len(ctxs) * 64, dtype=torch.uint8, device="cuda")
    flush = torch.empty(512 * 1024 * 1024, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.Stream()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]

    def launch(k):
        c = ctxs[k % len(ctxs)]
        c.launch(setups[k % len(ctxs)].seed, 15, hits.data_ptr(), cap,
                 counters.data_ptr() + 64 * (k % len(ctxs)), stream.cuda_stream)

    with torch.cuda.stream(stream):
        for k in range(args.warmup):
            flush.zero_()
            launch(k)
    torch.cuda.synchronize()

    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    wall0 = time.perf_counter()
    steps_taken = 0
    n_hits_total = 0
    with torch.cuda.stream(stream):
        for k in range(args.steps):
            flush.zero_()
            ev[k][0].record(stream)
            launch(k)
            ev[k][1].record(stream)
    torch.cuda.synchronize()
    wall = time.perf_counter() - wall0
    if world > 1:
        torch.distributed.barrier()
    clocks.stop()
    ms = [a.elapsed_time(b) for a, b in ev]
    cnt = counters.cpu().numpy().view(np.uint64).reshape(len(ctxs), 8)
    for k in range(args.steps):
        row = cnt[k % len(ctxs)]
        steps_taken += int(row[2])
        n_hits_total += int(row[0])
        assert int(row[4]) & 0xffffffff == 0, f"device error flags {row[4]}"
        assert int(row[1]) == photons_rank, (int(row[1]), photons_rank)
    kernel_s = sum(ms) / 1e3
    if world > 1:
        t = torch.tensor([kernel_s], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        kernel_s = float(t.item())
    value = photons_rank * world * args.steps / kernel_s
    ms_per_step = kernel_s * 1e3 / args.steps

    # roofline: FP32-issue bound
    peak = pp.measure_fp32_peak(local)
    # the photon steps of the last timed steps (counters of each context)
    flops = FLOPS_PER_STEP * steps_taken
    achieved = flops / kernel_s / 1e12
    traffic_full = profile_traffic()

    # e2e through the public API with host buffers
    e2e_steps = args.e2e_steps or min(args.steps, 3)
    hb = pp.HitBuffers(cap, local)
    for s in setups:
        if world > 1:
            s.sources = shard_sources(s, rank, world)
    if tuning is not None:  # the same autotuner, run once through the public API
        pp.autotune(setups[0], 15, sample_photons=min(photons, 8_000_000), device=local)
    pp.propagate_photons(setups[0], hb)  # warm (uploads this setup)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    h2d = d2h = 0
    e2e_photons = 0
    for k in range(e2e_steps):
        s = setups[k % len(setups)]
        t = pp.propagate_photons(s, hb)
        e2e_photons += sum(pp.source_photons(x.photons, s.photon_scaling) for x in s.sources)
        h2d += 96 * len(s.sources) + 24 * len(s.sources) + 8
        d2h += 48 + 80 * t.nrow
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    if world > 1:  # the slowest rank's time, as for the kernel
        t = torch.tensor([e2e_s], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        e2e_s = float(t.item())
    e2e_value = e2e_photons * world / e2e_s
    c2 = None if (world > 1 or args.no_c2 or args.config != "c1") else bench_c2(pp, torch, local)
    c0 = None if (world > 1 or args.no_c0) else bench_c0(pp, torch, local)
    refalg = None if (world > 1 or args.no_proxy or args.config != "c1") else \
        bench_reference_algorithm_gpu(pp, torch, local, value)
    sur = None if (world > 1 or args.no_surrogate) else bench_surrogate(pp, torch, local, args)
    detection = None if (world > 1 or args.no_detection) else bench_detection(
        pp, torch, local, n=int(args.detection_records))

    if rank != 0:
        return 0
    orc = entry.load_oracle()
    orc.build()
    base = cpu_baseline(pp, orc, args.config, args.cpu_seconds, photons)
    tun = ctxs[0].get_tuning()
    gi = ctxs[0].grid_info()
    line = {
        "metric": "photons/s on 1 GB300", "value": value, "unit": "photons/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {
            "workload": workload_name(args.config),
            "photons_per_step": photons, "seeds": [1, 2, 3, 4, 5],
            "l2": "flushed between steps (512 MiB write)",
            "tuning": {"block_threads": tun.block_threads,
                       "photons_per_thread": tun.photons_per_thread,
                       "cell_size_m": round(float(tun.cell_size or gi["cell"][0]), 3),
                       "grid_cells": gi["dims"], "autotuned": tuning is not None},
            "parallelism": f"photon-range shards x{world}" if world > 1 else "single GPU",
        },
        "e2e": {"value": e2e_value, "unit": "photons/s", "h2d_bytes_per_step": h2d // e2e_steps,
                "d2h_bytes_per_step": d2h // e2e_steps, "steps": e2e_steps,
                "api": "propagate_photons(setup, hit_buffers) -> hit table in host memory"
                       + (" (context tuned once by pp.autotune(setup))" if tuning else "")},
        "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak,
                     "traffic": traffic_full,
                     "issue_active_frac_ncu": profile_value("issue_active_frac"),
                     "note": f"{FLOPS_PER_STEP} algorithmic FP32 ops per photon step x "
                             f"{steps_taken / args.steps:.4g} steps per launch (device counter); "
                             "peak = measured FFMA throughput of this GPU (pp_measure_fp32_peak)"},
        "hits_per_step": n_hits_total / args.steps,
        "photon_steps_per_step": steps_taken / args.steps,
        "hit_write_gbs": n_hits_total * 80 / kernel_s / 1e9,
        "cpu_baseline": base,
        "clocks": clocks.summary(),
        "gpu_launches": args.steps,
        "c2_batched": c2,
        "c0": c0,
        "reference_algorithm_gpu": refalg,
        "surrogate": sur,
        "detection": detection,
        "wall_s_timed_region": wall,
    }
    print(json.dumps(line))
    return 0


def main():
    args = parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.surrogate_only:
        import torch
        _, _, local = dist_env()
        torch.cuda.set_device(local)
        print(json.dumps({"surrogate": bench_surrogate(entry.load(), torch, local, args)}))
        return 0
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
