#!/usr/bin/env python
"""Benchmark of the GB300 Gofrt engine on the 16k-atom workload.

Workload (the reference's headline configuration for this path): N=16384
atoms in 3 types (16352/16/16), cubic box at density 0.1 (L=54.72 A),
Gaussian random walk sigma=0.08 A, T=2000 frames; Gofrt(rmin=0, rmax=12,
nbin=400, tmax=200, skip=4), reset(1800), i.e. 450 origins x 200 lags x N^2
ordered pairs = 2.42e13 pair evaluations.  Seeded synthetic data
(analisi_gb300.workloads.c2), no dataset.

One step = one Gofrt::calculate over a window of 50 consecutive origins
(reset(200), calculate(primo)) x all 200 lags (2.68e12 ordered pairs; the
lags of a calculate are min(reset length, tmax), so the window must be at
least tmax frames long): step s uses primo=200*(s mod 9), so 9 steps are
exactly the full reset(1800) calculation, split the way the reference's
block-average driver splits a trajectory.

  value   pair throughput with the frames resident in HBM (device-timed with
          CUDA events on the engine's stream, L2 flushed between steps).
          Pairs are the reference's: N^2 ordered pairs per (lag, origin).
          The engine's default (auto) plan may take the cell-list kernel,
          which evaluates only the pairs of neighbouring cells (the others
          are provably beyond rmax); the counts are identical, so the value
          is the all-pairs-equivalent rate, and config.evaluated_frac says
          what share of the pairs was evaluated
  e2e     the same metric through the C ABI with host buffers: every step
          uploads its 400-frame window from pinned host memory
          (gofr_set_frames) and reads the counts back (gofr_run)
  roofline  FP32-issue bound: 16 FP32 lane operations per ordered pair of
          the reference loop (all N^2 pairs, orthorhombic minimum image) per
          mean kernel time, against the FP32 lane-op peak measured on this GPU
          by gofr_measure_peaks; beside it the kernel's own issue rate over
          the pairs it evaluated (7 operations each in the cell-list kernel)
  cpu_baseline  the C restatement of the reference (oracle/gofr_oracle.c,
          same fork/join thread split as the reference) on this host's cores,
          on a bounded sample of the same workload

--impl reference times that CPU implementation alone (the reference's own
algorithm on the host cores), with the same metric and configuration.
"""
import argparse
import json
import os
import re
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "g(r,t) Gpairs/s on 1 GB300: FP32+FP64-edge-recheck vs plain FP64, exact counts"
UNIT = "Gpairs/s"
ORIGINS_PER_STEP = 50
STEP_WINDOWS = 9  # windows of ORIGINS_PER_STEP origins in reset(1800)
OPS_PER_PAIR = 16  # orthorhombic FP32 pair: 3 sub + 3x(ffma, fadd, ffma) + fmul + 2 ffma + cmp
OPS_PER_PAIR_CELL = 7  # cell-list pair, images pre-shifted: 3 sub + fmul + 2 ffma + cmp
OPS_PER_PAIR_TRI = 19  # triclinic FP32 pair: 3 sub + wrap z (5), y (4), x (3) + 3 for d2 + cmp


def _measured_hbm_gbs():
    """Copy bandwidth of MEASURED_PEAKS.json (GB/s), if the file is there."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"])
    except (OSError, KeyError, ValueError):
        return None


HBM_GBS = _measured_hbm_gbs()


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-f64", action="store_true")
    ap.add_argument("--workload", default="c2",
                    choices=["c2", "batch", "cells", "tric", "msd", "neigh"],
                    help="c2: the headline line (default); batch / cells: only that measurement")
    ap.add_argument("--batch-origins", type=int, default=0,
                    help="origins per trajectory of the batched measurement (0: every origin "
                         "of the workload, stride 5)")
    ap.add_argument("--kernel", default="auto", choices=["auto", "f32", "cell", "tuned"],
                    help="pair kernel of the headline line (auto: what a user gets)")
    ap.add_argument("--no-extra", action="store_true",
                    help="skip the batched (64 trajectories) and cell-list (131k atoms) lines")
    ap.add_argument("--lags", type=int, default=200,
                    help="tmax of every step (200 = the workload; smaller only for ncu captures)")
    return ap.parse_args()


def dist_info():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def max_over_ranks(v, world):
    """The largest of every rank's v (the job's time is its slowest rank's)."""
    if world <= 1:
        return v
    import torch
    t = torch.tensor([float(v)], dtype=torch.float64)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t[0])


def step_window(s, rank=0):
    """primo of step s: 9 windows of 200 origin-frames cover reset(1800)."""
    return 200 * ((s + rank * 4) % STEP_WINDOWS)


def workload_config(extra=None):
    cfg = {"workload": "c2_n16384_t2000_ortho", "natoms": 16384, "types": [16352, 16, 16],
           "box": "cubic L=54.72 (density 0.1)", "frames": 2000, "sigma": 0.08,
           "rmin": 0.0, "rmax": 12.0, "nbin": 400, "tmax": 200, "skip": 4, "every": 1,
           "reset": 1800, "step": "calculate over 50 origins (reset(200), primo=200*(s%9)) "
                                   "x 200 lags = 2.68e12 pairs; 9 steps = the full reset(1800)",
           "l2": "flushed between timed steps (256 MiB write); per-step inputs ~79 MB < L2"}
    if extra:
        cfg.update(extra)
    return cfg


# ---------------------------------------------------------------------------
# CPU leg: the oracle port with the reference's thread split
# ---------------------------------------------------------------------------
def cpu_sample(w, seconds=15.0, threads=None):
    """Times the C restatement on a bounded sample of the workload.
    Returns (Gpairs/s, threads, description)."""
    from oracle import oracle
    oracle.build()
    threads = threads or os.cpu_count() or 1
    N = w["positions"].shape[1]
    p = w["params"]
    pos, boxes, tids = w["positions"], w["boxes"], w["type_ids"]

    def run(n_lags):
        # 1 origin, lags 0..n_lags-1: reset(n) with tmax=n and skip=n
        t0 = time.perf_counter()
        oracle.gofrt_counts(pos, boxes, tids, w["ntypes"], p["rmin"], p["rmax"], p["nbin"],
                            n_lags, threads, n_lags, 1, n_lags, 0)
        return time.perf_counter() - t0

    dt = run(1)
    n_lags = max(1, min(200, int(seconds / max(dt, 1e-3))))
    dt = run(n_lags)
    pairs = n_lags * N * N
    desc = (f"1 origin x {n_lags} lags of the workload ({pairs:.3g} ordered pairs), "
            f"{threads} threads forked/joined per (lag, origin) as the reference does")
    return pairs / dt / 1e9, threads, desc, dt


def run_reference(args):
    rank, world, _ = dist_info()
    if rank != 0:
        return 0
    from analisi_gb300 import workloads
    w = workloads.c2()
    from oracle import oracle
    oracle.build()
    threads = os.cpu_count() or 1
    N = 16384
    p = w["params"]
    n_lags = None
    times = []
    for s in range(args.warmup + args.steps):
        if n_lags is None:
            t0 = time.perf_counter()
            oracle.gofrt_counts(w["positions"], w["boxes"], w["type_ids"], w["ntypes"],
                                p["rmin"], p["rmax"], p["nbin"], 1, threads, 1, 1, 1, 0)
            dt1 = time.perf_counter() - t0
            n_lags = max(1, min(200, int(6.0 / max(dt1, 1e-3))))
        primo = step_window(s)
        t0 = time.perf_counter()
        oracle.gofrt_counts(w["positions"], w["boxes"], w["type_ids"], w["ntypes"], p["rmin"],
                            p["rmax"], p["nbin"], n_lags, threads, n_lags, 1, n_lags, primo)
        dt = time.perf_counter() - t0
        if s >= args.warmup:
            times.append(dt)
    pairs = n_lags * N * N
    val = pairs * len(times) / sum(times) / 1e9
    from oracle.oracle import host_info
    hi = host_info()
    sample = (f"each step: 1 origin (primo=200*(s%9)) x {n_lags} lags = {pairs:.3g} pairs "
              f"on {threads} threads of {hi['cpu']} ({hi['arch']})")
    out = {"metric": METRIC, "value": round(val, 4), "unit": UNIT, "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": round(1e3 * sum(times) / len(times), 3), "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "impl": "reference",
           "config": workload_config({"reference_kind": "port of lib/src/gofrt.cpp "
                                      "(oracle/gofr_oracle.c): the reference's sources need "
                                      "its tree, absent on this host"}),
           "cpu_baseline": {"value": round(val, 4), "unit": UNIT, "cores": threads,
                            "kind": "port", "sample": sample},
           "e2e": {"value": round(val, 4), "unit": UNIT, "h2d_bytes_per_step": 0,
                   "d2h_bytes_per_step": 0}}
    print(json.dumps(out))
    return 0


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
class Clocks:
    def __init__(self, path):
        self.path = path
        self.proc = None

    def __enter__(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "--query-gpu=index,clocks.sm,clocks.max.sm,power.draw,"
                 "clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
                 "clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.f, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.f.close()

    def summary(self, gpu_index):
        try:
            rows = [l.split(",") for l in open(self.path) if l.strip()]
        except OSError:
            return None
        rows = [[c.strip() for c in r] for r in rows if len(r) >= 9]
        rows = [r for r in rows if r[0] == str(gpu_index)] or rows
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if re.match(r"^[\d.]+$", r[1])]
        mx = [float(r[2]) for r in rows if re.match(r"^[\d.]+$", r[2])]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for k, n in enumerate(names):
                if r[5 + k].lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(rows)}


KERNEL_NAMES = {1: "k_pairs_f32 (all pairs)", 2: "k_pairs_f64 (all pairs)",
                3: "k_pairs_cell (block cell lists)",
                5: "k_pairs_cellw (warp-streamed cell lists)"}
PROFILE_OF = {1: "k_pairs_f32_c2_n16384.md", 3: "k_pairs_cell_c2_n16384.md",
              5: "k_pairs_cellw_c2_n16384.md"}


def traffic_from_profiles(kernel_used):
    """dram bytes per launch of the pair kernel from the committed ncu summary."""
    if kernel_used not in PROFILE_OF:
        return None
    path = os.path.join(ROOT, "profiles", PROFILE_OF[kernel_used])
    try:
        for line in open(path):
            m = re.search(r"traffic_bytes_per_launch:\s*([\d.eE+]+)", line)
            if m:
                return float(m.group(1))
    except OSError:
        pass
    return None


def bench_batch(engine, workloads, device, origins=0, reps=2):
    """The 64 uneven trajectories (seeds 2000+k) in one graph-captured batch:
    the members the planner gives cell lists run the warp-streamed cell-list
    kernel (one launch each, on a second stream), the rest share one
    persistent all-pairs launch with a device work queue.  Against the same
    trajectories run one by one with the same plans.  origins=0: every origin
    of every member (stride 5, lags up to min(100, T/2)), as the workload
    states; the all-pairs comparison runs on 20 origins per member."""
    import numpy as np
    mem = workloads.c4(64)

    def params_of(m, n_orig):
        p = m["params"]
        n = p["ntimesteps"] if not n_orig else min(p["ntimesteps"], n_orig * p["skip"])
        return engine.make_params(p["rmin"], p["rmax"], p["nbin"], p["tmax"], p["skip"],
                                  p["every"], n, 0)

    trajs = [dict(positions=m["positions"], boxes=m["boxes"], type_ids=m["type_ids"],
                  ntypes=m["ntypes"], params=params_of(m, origins)) for m in mem]
    e = engine.Engine(device)
    e.batch_set(trajs)
    outs = e.batch_run(use_graph=True)  # warm-up (graph capture)
    ms = []
    for _ in range(reps):
        e.batch_run(use_graph=True)
        ms.append(e.stats()["kernel_ms"])
    st = e.stats()
    batch_rate = st["pairs"] / (sum(ms) / len(ms)) / 1e6
    e.close()
    # the same trajectories one by one: with the kernel a single run picks by
    # itself, and (on 20 origins each) with the all-pairs kernel
    seq = {}
    same = True
    e2 = engine.Engine(device)
    for kern, n_orig in (("auto", origins), ("f32", 20)):
        ms_sum, pairs_sum, best = 0.0, 0, 0.0
        for k, m in enumerate(mem):
            e2.set_frames(m["positions"], m["boxes"], m["type_ids"], m["ntypes"])
            P = params_of(m, n_orig)
            c = e2.run(P.rmin, P.rmax, P.nbin, P.tmax, P.skip, P.every, P.ntimesteps, P.primo,
                       kernel=kern)
            s2 = e2.stats()
            ms_sum += s2["kernel_ms"]
            pairs_sum += s2["pairs"]
            best = max(best, s2["pairs"] / s2["kernel_ms"] / 1e6)
            if kern == "auto":
                same &= bool(np.array_equal(c, outs[k]))
        seq[kern] = (pairs_sum / ms_sum / 1e6, best)
    e2.close()
    desc = "every origin (stride 5)" if not origins else f"{origins} origins"
    return {"workload": "64 trajectories, N log-uniform 256..16384, T 100..1000, 1-4 types, "
                        f"300 bins on [0,10], {desc} x lags up to min(100, T/2) each",
            "pairs": st["pairs"], "value": round(batch_rate, 2), "unit": UNIT,
            "ms": round(sum(ms) / len(ms), 1),
            "kernel": "one graph: k_pairs_cellw per cell-list member (second stream) + "
                      "k_pairs_batch (all-pairs members, persistent work queue)",
            "evaluated_fraction": round(st["evaluated"] / st["pairs"], 4),
            "sequential_same_plans": round(seq["auto"][0], 2),
            "best_single_same_plans": round(seq["auto"][1], 2),
            "ratio_vs_sequential": round(batch_rate / seq["auto"][0], 3),
            "ratio_vs_best_single": round(batch_rate / seq["auto"][1], 3),
            "sequential_all_pairs_kernel_20_origins": round(seq["f32"][0], 2),
            "best_single_all_pairs_kernel_20_origins": round(seq["f32"][1], 2),
            "counts_identical_to_single_runs": same, "cuda_graph": True}


def bench_allpairs(eng, prm, args, flush, steps=2):
    """The same steps through the all-pairs FP32 kernel (for comparison when the
    headline line used the cell-list form)."""
    import numpy as np
    import torch
    from analisi_gb300 import engine
    pairs, ms = 0, 0.0
    for s in range(steps + 1):
        p = prm[(args.warmup + s) % STEP_WINDOWS]
        q = engine.make_params(p.rmin, p.rmax, p.nbin, p.tmax, p.skip, p.every, p.ntimesteps,
                               p.primo, kernel="f32")
        out = np.zeros(eng.output_size(q), dtype=np.uint64)
        flush.zero_()
        torch.cuda.synchronize()
        eng.run_params(q, out)
        st = eng.stats()
        if s > 0:
            pairs += st["pairs"]
            ms += st["kernel_ms"]
    return {"value": round(pairs / ms / 1e6, 3), "unit": UNIT, "steps": steps,
            "kernel": "k_pairs_f32 (all pairs)"}


def bench_msd(eng, w, p, reps=3):
    """MeanSquareDisplacement on the same resident 16k-atom frames, the job of
    the g(r,t) headline (reset(1800), tmax=200, skip=4: 450 origins x 200 lags
    x 16384 atoms = 1.47e9 squared displacements), both centre-of-mass options
    on; checked against the oracle's running means on a sub-sample, and the
    oracle (one thread) timed on a bounded sample of the same job."""
    import numpy as np
    from oracle import oracle
    N = w["positions"].shape[1]
    nt = w["ntypes"]
    cm = oracle.centres(w["positions"], w["type_ids"], nt)
    eng.set_centres(cm)
    eng.msd(p["skip"], p["tmax"], 1800, 0, True, True)
    ms = []
    for _ in range(reps):
        eng.msd(p["skip"], p["tmax"], 1800, 0, True, True)
        ms.append(eng.stats()["kernel_ms"])
    disp = 200 * 450 * N
    rate = disp / (sum(ms) / len(ms)) / 1e6
    # sub-sample check: 20 lags x 10 origins
    sub_gpu = eng.msd(p["skip"], 20, 40, 0, True, True)
    t0 = time.perf_counter()
    sub_ref = oracle.msd(w["positions"], w["type_ids"], nt, p["skip"], 20, 40, 0, True, True,
                         cm=cm)
    dt = time.perf_counter() - t0
    rel = float(np.max(np.abs(sub_gpu - sub_ref) / np.maximum(np.abs(sub_ref), 1e-300)))
    cpu_rate = 20 * 10 * N / dt / 1e9
    return {"workload": "c2 frames: reset(1800), tmax=200, skip=4, both centre-of-mass options",
            "displacements": disp, "ms": round(sum(ms) / len(ms), 3),
            "value": round(rate, 2), "unit": "G squared displacements/s",
            "fp64_ops_per_displacement": 9,
            "max_rel_diff_vs_oracle_sample": rel,
            "cpu_oracle_1thread": {"value": round(cpu_rate, 4), "unit": "G squared displacements/s",
                                   "sample": "20 lags x 10 origins", "seconds": round(dt, 3)}}


def bench_neigh(eng, w, frames=3):
    """Neighbours::update_neigh on frames of the resident 16k-atom trajectory:
    3 types, cutoff 3.5 (about 18 neighbours per type and atom), sorted lists; the
    oracle (one thread, the reference's i < j loop) timed on one frame of the
    first 2048 atoms, compared per pair."""
    import numpy as np
    from oracle import oracle
    spec = [(64, 3.5 ** 2, 4.0 ** 2)] * w["ntypes"]
    eng.neighbours(0, spec, True)
    ms = []
    for f in range(1, 1 + frames):
        eng.neighbours(f, spec, True)
        ms.append(eng.stats()["kernel_ms"])
    N = w["positions"].shape[1]
    n_sub = 2048
    t0 = time.perf_counter()
    oracle.neighbours(w["positions"][:2, :n_sub], w["boxes"][:2], w["type_ids"][:n_sub],
                      w["ntypes"], 1, spec, True)
    dt = time.perf_counter() - t0
    cpu_pairs_per_s = n_sub * (n_sub - 1) / 2 / dt
    gpu_frame_ms = sum(ms) / len(ms)
    return {"workload": "c2 frames (N=16384, 3 types), cutoff 3.5 for every type, sorted",
            "ms_per_frame": round(gpu_frame_ms, 3),
            "value": round(N * (N - 1) / 2 / (gpu_frame_ms * 1e-3) / 1e9, 3),
            "unit": "G atom pairs (i<j)/s",
            "cpu_oracle_1thread": {"value": round(cpu_pairs_per_s / 1e9, 4),
                                   "unit": "G atom pairs (i<j)/s",
                                   "sample": f"one frame of the first {n_sub} atoms",
                                   "seconds": round(dt, 3)}}


def bench_cells(engine, workloads, device):
    """131072 atoms, 4 types, 250 bins on [0,10]: the default plan (the
    warp-streamed cell-list kernel) and the block cell-list kernel on a sample
    (10 origins x 50 lags), their counts checked against each other and, on a
    sub-sample (1 origin x 5 lags), against the all-pairs FP32 kernel."""
    import numpy as np
    w = workloads.c5(T=150)
    p = w["params"]
    e = engine.Engine(device)
    e.set_frames(w["positions"], w["boxes"], w["type_ids"], w["ntypes"])
    res = {}
    for kern in ("auto", "cell"):
        for _ in range(2):
            c = e.run(p["rmin"], p["rmax"], p["nbin"], 50, p["skip"], 1, 100, 0, kernel=kern)
        res[kern] = (c, e.stats())
    st = res["auto"][1]
    a = e.run(p["rmin"], p["rmax"], p["nbin"], 5, p["skip"], 1, 5, 0)
    b = e.run(p["rmin"], p["rmax"], p["nbin"], 5, p["skip"], 1, 5, 0, kernel="f32")
    sf = e.stats()
    e.close()
    sc = res["cell"][1]
    return {"workload": "c5: N=131072, 4 types, L=109.47, rmax=10, 250 bins; 10 origins x 50 lags",
            "value": round(st["pairs"] / st["kernel_ms"] / 1e6, 1),
            "unit": UNIT + " (all-pairs equivalent)",
            "kernel": KERNEL_NAMES.get(st["kernel_used"], str(st["kernel_used"])),
            "evaluated_gpairs_per_s": round(st["evaluated"] / st["kernel_ms"] / 1e6, 1),
            "evaluated_fraction": round(st["evaluated"] / st["pairs"], 5),
            "block_cell_kernel_gpairs_per_s": round(sc["pairs"] / sc["kernel_ms"] / 1e6, 1),
            "block_cell_evaluated_fraction": round(sc["evaluated"] / sc["pairs"], 5),
            "all_pairs_f32_gpairs_per_s": round(sf["pairs"] / sf["kernel_ms"] / 1e6, 1),
            "counts_identical_block_vs_warp": bool(np.array_equal(res["auto"][0],
                                                                  res["cell"][0])),
            "counts_identical_to_all_pairs": bool(np.array_equal(a, b))}


def bench_triclinic(engine, workloads, device, peak):
    """32768 atoms in the triclinic cell a=(L,0,0), b=(0.3L,L,0), c=(0.2L,0.1L,L),
    L=70, 500 bins on [0,15]: the default plan (the warp-streamed cell-list
    kernel on the tilted cell) and the all-pairs FP32 kernel with the
    triclinic minimum image on a sample of 10 origins x 20 lags, their counts
    checked against each other and, on 1 origin x 2 lags, against the plain
    FP64 kernel."""
    import numpy as np
    w = workloads.c3(T=80)
    p = w["params"]
    e = engine.Engine(device)
    e.set_frames(w["positions"], w["boxes"], w["type_ids"], w["ntypes"])
    res = {}
    for kern in ("auto", "f32"):
        for _ in range(2):
            c = e.run(p["rmin"], p["rmax"], p["nbin"], 20, p["skip"], 1, 50, 0, kernel=kern)
        res[kern] = (c, e.stats())
    st, sa = res["auto"][1], res["f32"][1]
    a = e.run(p["rmin"], p["rmax"], p["nbin"], 2, p["skip"], 1, 1, 0)
    b = e.run(p["rmin"], p["rmax"], p["nbin"], 2, p["skip"], 1, 1, 0, kernel="f64")
    sf = e.stats()
    e.close()
    rate = st["pairs"] / st["kernel_ms"] / 1e6
    rate_ap = sa["pairs"] / sa["kernel_ms"] / 1e6
    out = {"workload": "c3: N=32768, triclinic (0.3L, 0.2L, 0.1L tilts), L=70, rmax=15, 500 bins; "
                       "10 origins x 20 lags",
           "value": round(rate, 1), "unit": UNIT + " (all-pairs equivalent)",
           "kernel": KERNEL_NAMES.get(st["kernel_used"], str(st["kernel_used"])),
           "evaluated_gpairs_per_s": round(st["evaluated"] / st["kernel_ms"] / 1e6, 1),
           "evaluated_fraction": round(st["evaluated"] / st["pairs"], 5),
           "all_pairs_f32_gpairs_per_s": round(rate_ap, 1),
           "fp32_ops_per_pair_all_pairs": OPS_PER_PAIR_TRI,
           "f64_kernel_gpairs_per_s": round(sf["pairs"] / sf["kernel_ms"] / 1e6, 2),
           "counts_identical_warp_vs_all_pairs": bool(np.array_equal(res["auto"][0],
                                                                     res["f32"][0])),
           "counts_identical_to_f64": bool(np.array_equal(a, b))}
    if peak:
        out["all_pairs_roofline_frac"] = round(rate_ap * 1e9 * OPS_PER_PAIR_TRI / (peak * 1e12), 3)
    return out


def run_gpu(args):
    import numpy as np
    import torch
    rank, world, local = dist_info()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    torch.cuda.set_device(local)
    from analisi_gb300 import engine, workloads
    w = workloads.c2()
    p = w["params"]
    N = w["positions"].shape[1]
    eng = engine.Engine(local)
    eng.set_frames(w["positions"], w["boxes"], w["type_ids"], w["ntypes"])
    step_n = ORIGINS_PER_STEP * p["skip"]
    lags = min(args.lags, p["tmax"])
    prm = [engine.make_params(p["rmin"], p["rmax"], p["nbin"], lags, p["skip"], p["every"],
                              step_n, step_window(s, rank), kernel=args.kernel)
           for s in range(STEP_WINDOWS)]
    nout = eng.output_size(prm[0])
    out = np.zeros(nout, dtype=np.uint64)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{local}")

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()

    # warm-up
    for s in range(args.warmup):
        eng.run_params(prm[s % STEP_WINDOWS], out)
    st0 = eng.stats()
    launches0 = st0["launches"]
    kernel_ms, total_ms, cands, rech, pairs, evaluated = [], [], 0, 0, 0, 0
    kernels_used = set()
    barrier()
    # raw clock samples of the timed region (the JSON line carries their summary)
    out_dir = os.environ.get("ANALISI_GB300_BENCH_OUT", os.path.join(ROOT, "bench_out"))
    os.makedirs(out_dir, exist_ok=True)
    with Clocks(os.path.join(out_dir, f"clocks_rank{rank}.csv")) as clk:
        for s in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            eng.run_params(prm[(args.warmup + s) % STEP_WINDOWS], out)
            st = eng.stats()
            kernel_ms.append(st["kernel_ms"])
            total_ms.append(st["total_ms"])
            cands += st["candidates"]
            rech += st["rechecks"]
            pairs += st["pairs"]
            evaluated += st["evaluated"]
            kernels_used.add(int(st["kernel_used"]))
    barrier()
    launches = eng.stats()["launches"] - launches0
    dev_s = max_over_ranks(sum(total_ms) / 1e3, world)
    value = pairs * world / dev_s / 1e9
    kernel_avg_s = sum(kernel_ms) / len(kernel_ms) / 1e3
    pairs_per_launch = pairs / args.steps

    # e2e through the C ABI with host buffers (pinned), copies in the timed region
    e2e = None
    if not args.no_e2e:
        win_frames = step_n + p["tmax"]
        pinned_pos = torch.empty((win_frames, N, 3), dtype=torch.float64).pin_memory()
        pinned_box = torch.empty((win_frames, 6), dtype=torch.float64).pin_memory()
        pp, pb = pinned_pos.numpy(), pinned_box.numpy()
        e2 = engine.Engine(local)
        pe = [engine.make_params(p["rmin"], p["rmax"], p["nbin"], lags, p["skip"],
                                 p["every"], step_n, 0, kernel=args.kernel) for _ in range(1)]
        times = []
        h2d = win_frames * N * 24 + win_frames * 48 + N * 4
        for s in range(args.warmup + args.steps):
            primo = step_window(s, rank)
            pp[...] = w["positions"][primo:primo + win_frames]
            pb[...] = w["boxes"][primo:primo + win_frames]
            flush.zero_()
            barrier()
            t0 = time.perf_counter()
            e2.set_frames(pp, pb, w["type_ids"], w["ntypes"])
            e2.run_params(pe[0], out)
            dt = time.perf_counter() - t0
            if s >= args.warmup:
                times.append(dt)
        e2_launch = e2.stats()["launches"]
        e2.close()
        e2e_s = max_over_ranks(sum(times), world)
        e2e = {"value": round(pairs * world / e2e_s / 1e9, 3), "unit": UNIT,
               "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(nout * 8),
               "timing": "host wall clock around gofr_set_frames + gofr_run (synchronous)",
               "launches": int(e2_launch)}

    # FP64 comparison kernel on a sample (1 origin x 10 lags), same engine
    f64 = None
    if rank == 0 and not args.no_f64:
        pf = engine.make_params(p["rmin"], p["rmax"], p["nbin"], 10, 10, p["every"],
                                10, 0, kernel="f64")
        o64 = np.zeros(eng.output_size(pf), dtype=np.uint64)
        eng.run_params(pf, o64)
        st = eng.stats()
        pf32 = engine.make_params(p["rmin"], p["rmax"], p["nbin"], 10, 10, p["every"],
                                  10, 0, kernel="f32")
        o32 = np.zeros_like(o64)
        eng.run_params(pf32, o32)
        st32 = eng.stats()
        f64 = {"gpairs_per_s_f64": round(st["pairs"] / st["kernel_ms"] / 1e6, 3),
               "gpairs_per_s_f32_same_sample": round(st32["pairs"] / st32["kernel_ms"] / 1e6, 3),
               "counts_identical": bool(np.array_equal(o64, o32)),
               "sample": "1 origin x 10 lags (2.68e9 pairs)"}

    if rank != 0:
        if world > 1:
            torch.distributed.barrier()
        return 0

    fp32_peak, satom_peak = engine.measure_peaks(local)
    kernel_used = max(kernels_used) if kernels_used else 0
    evaluated_per_launch = evaluated / args.steps
    ops_eval = OPS_PER_PAIR_CELL if kernel_used in (3, 5) else OPS_PER_PAIR
    peak = fp32_peak / 1e12
    # the unit of the metric: every ordered pair of the reference loop at the
    # all-pairs kernel's 16 FP32 operations (orthorhombic minimum image)
    achieved = pairs_per_launch * OPS_PER_PAIR / kernel_avg_s / 1e12
    # what the kernel itself issued: its evaluated pairs at its own cost
    achieved_eval = evaluated_per_launch * ops_eval / kernel_avg_s / 1e12
    traffic = traffic_from_profiles(kernel_used)
    # algorithmic bytes: each (origin, lag) item reads two FP32 frames
    # (N x 12 B each); the items of one launch
    items_per_launch = ORIGINS_PER_STEP * lags
    algo_bytes = items_per_launch * 2 * N * 12
    roof = {"bound": "fp32", "achieved": round(achieved, 3), "peak": round(peak, 3),
            "unit": "TFLOP/s", "frac": round(achieved / peak, 4),
            "traffic": traffic,
            "peak_source": "gofr_measure_peaks: FFMA issue rate measured on this GPU (burst); "
                           "MEASURED_PEAKS.json holds no FP32 peak",
            "notes": "achieved = 16 FP32 lane operations (one FADD/FMUL/FFMA = 1) x every "
                     "ordered pair of the reference loop (N^2 per origin and lag) / mean kernel "
                     "time: the all-pairs unit of the metric.  The cell-list kernel evaluates "
                     "only the pairs of neighbouring cells at 7 operations each (three "
                     "differences, a multiply, two FMAs, the candidate test; neighbours moved "
                     "to their image once per chunk); frac_evaluated_pairs is that issue rate "
                     "against the same peak.  Candidate binning is counted in neither.  "
                     "traffic = ncu dram bytes per launch (profiles/)",
            "frac_evaluated_pairs": round(achieved_eval / peak, 4),
            "achieved_evaluated_pairs": round(achieved_eval, 3),
            "ops_per_evaluated_pair": ops_eval,
            "kernel": KERNEL_NAMES.get(kernel_used, str(kernel_used)),
            "pairs_per_launch": int(pairs_per_launch),
            "evaluated_pairs_per_launch": int(evaluated_per_launch),
            "algorithmic_bytes_per_launch": int(algo_bytes),
            "traffic_over_algorithmic_bytes": (round(traffic / algo_bytes, 1)
                                               if traffic else None),
            "hbm_frac_of_measured": (round(traffic / kernel_avg_s / 1e9 / HBM_GBS, 4)
                                     if traffic and HBM_GBS else None),
            "smem_atomic_peak_per_s": satom_peak,
            "atomics_needed_per_s": round(cands / (sum(kernel_ms) / 1e3), 1),
            # the all-pairs bound: every N^2 pair at 16 FP32 operations and the
            # measured peak (frac above is the kernel's rate against it)
            "allpairs_bound_gpairs_per_s": round(fp32_peak / OPS_PER_PAIR / 1e9, 1)}
    cpu = None
    if not args.no_cpu_baseline:
        v, thr, desc, dt = cpu_sample(w, seconds=15.0)
        cpu = {"value": round(v, 4), "unit": UNIT, "cores": thr, "kind": "port",
               "sample": desc, "seconds": round(dt, 2)}
    clocks = clk.summary(local)
    extra = {}
    if not args.no_extra:
        extra["msd"] = bench_msd(eng, w, p)
        extra["neighbours"] = bench_neigh(eng, w)
        del w
        if kernel_used != 1:
            extra["allpairs_f32"] = bench_allpairs(eng, prm, args, flush)
        extra["batch64"] = bench_batch(engine, workloads, local, args.batch_origins)
        extra["cells131k"] = bench_cells(engine, workloads, local)
        extra["triclinic32k"] = bench_triclinic(engine, workloads, local,
                                                roof.get("peak") if roof else None)
    res = {"metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": world,
           "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": round(1e3 * dev_s / args.steps, 3), "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64-recheck (u64 counts)",
           "data": "synthetic (seeded random walk, analisi_gb300.workloads.c2)",
           "config": workload_config({"pairs_per_step": int(pairs_per_launch), "lags": lags,
                                      "kernel": KERNEL_NAMES.get(kernel_used, str(kernel_used)),
                                      "kernel_request": args.kernel,
                                      "evaluated_frac": round(evaluated / pairs, 6),
                                      "candidates_frac": round(cands / pairs, 6),
                                      "recheck_frac": rech / pairs}),
           "e2e": e2e, "gpu_launches": int(launches), "roofline": roof, "cpu_baseline": cpu,
           "clocks": clocks, "fp64_kernel": f64, **extra,
           "kernel_ms_per_step": round(1e3 * kernel_avg_s, 3),
           # (origin, lag) items of all ranks per second (frames compared per second)
           "items_per_s": round(world * ORIGINS_PER_STEP * lags * args.steps / dev_s, 1)}
    print(json.dumps(res))
    if world > 1:
        torch.distributed.barrier()
    return 0


def run_one(args):
    """One secondary measurement alone (for profiling captures)."""
    from analisi_gb300 import engine, workloads
    if args.workload == "batch":
        r = bench_batch(engine, workloads, 0, args.batch_origins, reps=max(1, args.steps))
    elif args.workload in ("msd", "neigh"):
        w = workloads.c2()
        eng = engine.Engine(0)
        eng.set_frames(w["positions"], w["boxes"], w["type_ids"], w["ntypes"])
        if args.workload == "msd":
            r = bench_msd(eng, w, w["params"], reps=max(1, args.steps))
        else:
            r = bench_neigh(eng, w, frames=max(1, args.steps))
        eng.close()
    elif args.workload == "tric":
        r = bench_triclinic(engine, workloads, 0, None)
    else:
        r = bench_cells(engine, workloads, 0)
    print(json.dumps(r))
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload != "c2":
        return run_one(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
