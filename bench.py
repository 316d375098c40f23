"""Benchmark of the GB300 INSCY engine on the 25,000 x 15 plain-GPU workload.

One step = one complete INSCY run (all lattice levels, clustering and the
ordered commit) over one synthetic dataset of the workload: n=25,000 float32
points in d=15 dims, 10 Gaussian clusters of 2,250 points (std 0.02) in
random 4-6 dim subspaces, 2,500 uniform noise points; neighborhood_size=0.03,
F=1, num_obj=4, min_size=16, r=1, number_of_cells=4.  The metric is points
clustered per second (n / run time) and ms per run.

  value   -- device-resident: X already in HBM, inscy_run_device, CUDA events on
             the engine's stream, L2 flushed (256 MiB write) before every step;
  e2e     -- the reference-facing call with host buffers (inscy_run: host X in,
             host labels out), host clock, copies included;
  roofline-- the density candidate pass (k_neighbours_rows, the dominant
             kernel; its level-1 counterpart is one of the averaged launches):
             algorithmic bytes per launch / its average launch time, against
             the measured HBM copy bandwidth; roofline_tree the same for the
             restrict/merge/prune level kernel (k_tree_level);
  parity  -- the timed run's labels against the oracle's on the same input
             (tests/golden/full_plain.json: per-subspace label digests made by
             the oracle restatement of the reference CPU INSCY);
  cpu_baseline -- the CPU restatement of the reference CPU INSCY (oracle/) on a
             bounded sample of the workload (its first 8,000 rows), all host
             cores.

batched -- the 64-dataset batch workload: plain runs one after another vs the
             batched form (concurrent lanes; the lane count timed among 2, 4
             and 8 on 24 of the datasets) with FIFO and with the learned
             schedule (cost model trained on the committed cost records),
             three alternating runs of each, the best counting; labels against
             the plain runs and the oracle fixtures of 8 datasets.
large_d -- the 100,000 x 25 workload, one warm-up run then one timed (e2e,
             host buffers), labels against its oracle fixture.
autotune -- the row kernel's launch shape the engine's tuner chose.
real_shapes -- e2e ms per run on stand-ins with the sizes of the reference's
             real-data runs and its real-data parameters, next to the wall
             times the reference publishes for GPU-INSCY on the real datasets
             (experiments/plot_real.py:14; other data, unstated hardware).

`--impl reference` times the reference's CPU INSCY path (the oracle port of
run_cpu3_weak, all host cores) on the full workload instead: one complete run
per step, as many steps (up to --steps) as fit in --ref-budget seconds.
Multi-GPU: replicas only (`--gpus N` under torchrun runs N independent copies
of the workload, one per GPU).
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

WORKLOAD = "plain_n25000_d15"  # the default; --n changes n for profiling captures
METRIC = "INSCY points/sec (plain GPU run, bit-exact labels)"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--n", type=int, default=25_000, help="points (profiling captures use a smaller case)")
    ap.add_argument("--cpu-sample", type=int, default=8000, help="rows of the workload the CPU baseline runs on")
    ap.add_argument("--ref-budget", type=float, default=240.0,
                    help="--impl reference: seconds of timed CPU runs (at least one full run)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batched", action="store_true", help="skip the batched / learned-schedule measurement")
    ap.add_argument("--no-extra", action="store_true", help="skip the large_d and real-shape measurements")
    return ap.parse_args()


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """nvidia-smi samples of SM clocks and throttle reasons during the timed region."""
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([v.strip() for v in line.split(",")])

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        sm = [float(r[0]) for r in self.rows if r and r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if len(r) > 1 and r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            for k, name in enumerate(names):
                if len(r) > 4 + k and r[4 + k].lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.rows)}


def measured_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def cpu_baseline(X, p, sample_rows):
    """Oracle port of the reference CPU INSCY on the first `sample_rows` rows
    (one run, all host cores)."""
    import oracle as orc
    Xs = np.ascontiguousarray(X[:sample_rows])
    cores = os.cpu_count() or 1
    orc.load()
    t0 = time.perf_counter()
    orc.run(Xs, **p, threads=cores)
    t = time.perf_counter() - t0
    return {"value": Xs.shape[0] / t, "unit": "points/s", "cores": cores, "kind": "port",
            "sample": "first %d of the %d rows of the %s workload, same parameters; %.2f s per run"
                      % (Xs.shape[0], X.shape[0], WORKLOAD, t)}


def fixture_check(name, subs, labels, index=None):
    """The CUDA path's output against an oracle fixture entry (True / False),
    or None when the fixture does not exist."""
    if os.path.join(ROOT, "tests") not in sys.path:
        sys.path.insert(0, os.path.join(ROOT, "tests"))
    from golden_io import GOLDEN, full_fixture, result_digest
    if not os.path.exists(os.path.join(GOLDEN, "full_%s.json" % name)):
        return None
    ents = full_fixture(name)["entries"]
    e = ents[0] if index is None else next((x for x in ents if x.get("index") == index), None)
    if e is None:
        return None
    g = result_digest(subs, labels)
    return g["subspaces"] == e["subspaces"] and g["label_sha256"] == e["label_sha256"]


def batched_block(_lib):
    """The batched form on the 64-dataset batch workload (seed 0, held out from
    the cost records): plain (sequential) vs concurrent lanes with the FIFO
    schedule vs the learned (longest predicted first) schedule; the lane
    count is autotuned on a subset."""
    from gpu_inscy_gb300 import scheduler, synth
    Xs = synth.make_batch(0)
    p = dict(synth.PARAMS["batch"])
    params = _lib.make_params(**p)
    points = int(sum(x.shape[0] for x in Xs))
    plain, t_plain = [], []
    for X in Xs:
        t0 = time.perf_counter()
        plain.append(_lib.run_host(X, params)[:2])
        t_plain.append(time.perf_counter() - t0)
    # cost model from the committed records (none of them from this batch)
    recs = scheduler.load_records()
    model = scheduler.CostModel(seed=0).fit([r["features"] for r in recs], [r["ms"] for r in recs])
    F = np.array([scheduler.features(X, **p) for X in Xs])
    pred = model.predict_ms(F)
    err = float(np.median(np.abs(np.log(pred) - np.log(1000.0 * np.asarray(t_plain)))))
    learned = scheduler.lpt_order(pred)
    # autotune the lane count on the first 24 datasets (12 and 16 lanes can
    # win on this subset and lose on the whole batch: the lanes' host threads
    # then compete with the commits' pools for the host cores)
    sub = Xs[:24]
    tried = {}
    for lanes in (2, 4, 8):
        _lib.run_batch(sub, params, _lib.MODE_BATCHED, lanes=lanes)  # warm the lanes' engines
        t0 = time.perf_counter()
        _lib.run_batch(sub, params, _lib.MODE_BATCHED, lanes=lanes)
        tried[lanes] = time.perf_counter() - t0
    lanes = min(tried, key=tried.get)
    _lib.run_batch(Xs, params, _lib.MODE_BATCHED, lanes=lanes)  # warm-up at the chosen lane count
    # the two schedules alternate, three runs each; the best run of each counts
    # (one run's makespan varies by a few per cent with the host's load)
    fifo_runs, learned_runs = [], []
    for _ in range(3):
        t0 = time.perf_counter()
        fifo = _lib.run_batch(Xs, params, _lib.MODE_BATCHED, lanes=lanes)
        fifo_runs.append(time.perf_counter() - t0)
        t0 = time.perf_counter()
        lrn = _lib.run_batch(Xs, params, _lib.MODE_BATCHED, order=learned, lanes=lanes)
        learned_runs.append(time.perf_counter() - t0)
    t_fifo, t_learned = min(fifo_runs), min(learned_runs)
    same = all(a[0] == b[0] and a[0] == c[0] and np.array_equal(np.asarray(a[1]), np.asarray(b[1])) and
               np.array_equal(np.asarray(a[1]), np.asarray(c[1])) for a, b, c in zip(plain, fifo, lrn))
    # the datasets with oracle fixtures (tests/golden/full_batch.json)
    checked = {}
    for i in range(len(Xs)):
        ok = fixture_check("batch", lrn[i][0], lrn[i][1], index=i)
        if ok is not None:
            checked[str(i)] = bool(ok)
    return {"workload": "batch64_seed0 (64 datasets, n log-uniform in [2000, 50000], d in [8, 20])",
            "datasets": len(Xs), "points": points, "lanes": lanes,
            "lanes_tried_s": {str(k): round(v, 3) for k, v in tried.items()},
            "plain_s": round(sum(t_plain), 3), "fifo_s": round(t_fifo, 3), "learned_s": round(t_learned, 3),
            "fifo_runs_s": [round(t, 3) for t in fifo_runs], "learned_runs_s": [round(t, 3) for t in learned_runs],
            "plain_points_per_s": points / sum(t_plain), "fifo_points_per_s": points / t_fifo,
            "learned_points_per_s": points / t_learned,
            "learned_vs_plain": sum(t_plain) / t_learned, "learned_vs_fifo": t_fifo / t_learned,
            "cost_model": {"records": len(recs), "median_abs_log_error": err,
                           "final_train_loss": float(model.loss_hist[-1])},
            "labels_equal_plain": bool(same), "labels_equal_oracle_fixtures": checked}


# GPU-INSCY wall times the reference publishes for its real datasets, in
# seconds (experiments/plot_real.py:14); the shapes are synth.REAL_SHAPES
REFERENCE_REAL_GPU_S = {"glass": 0.0615, "vowel": 0.0373, "pendigits": 3.037, "sky": 4.892}


def extra_blocks(_lib):
    """The 100,000 x 25 workload (one warm-up run, one timed), and the
    real-data shapes (e2e)."""
    from gpu_inscy_gb300 import synth
    out = {}
    X = synth.make_large_d(0)
    params = _lib.make_params(**synth.PARAMS["large_d"])
    _lib.run_host(X, params)  # warm-up: the first run at a new size grows the memory pools
    t0 = time.perf_counter()
    subs, labs, st = _lib.run_host(X, params)
    t = time.perf_counter() - t0
    out["large_d"] = {"workload": "large_d_n100000_d25 (seed 0)", "ms_per_run": 1000.0 * t,
                      "labels_equal_oracle_fixture": fixture_check("large_d", subs, labs),
                      "points_per_s": X.shape[0] / t, "clustered_subspaces": len(subs),
                      "subspaces_evaluated": int(st["subspaces"]), "candidates": int(st["candidates"]),
                      "breakdown_ms": {k: st[k] for k in ("ms_expand", "ms_density", "ms_tree", "ms_cluster",
                                                          "ms_replay", "ms_commit_tail", "ms_total")}}
    shapes = {}
    for name, (n, d, _) in synth.REAL_SHAPES.items():
        X = synth.make_real_shape(name, seed=0)
        params = _lib.make_params(**synth.real_params(n))
        _lib.run_host(X, params)  # warm-up
        times = []
        for _ in range(3):
            t0 = time.perf_counter()
            subs, _, _ = _lib.run_host(X, params)
            times.append(time.perf_counter() - t0)
        shapes[name] = {"n": n, "d": d, "ms_per_run": 1000.0 * float(np.mean(times)),
                        "clustered_subspaces": len(subs),
                        "reference_gpu_inscy_s_on_the_real_dataset": REFERENCE_REAL_GPU_S[name]}
    out["real_shapes"] = shapes
    return out


def run_reference(args, X, p):
    """The reference's CPU INSCY path (the oracle port of run_cpu3_weak, all
    host cores) on the full workload: one complete run per step; steps stop
    once --ref-budget seconds of runs are done (at least one).  A CPU run has
    nothing to warm up beyond building the port, which happens first."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    import oracle as orc
    orc.load()
    cores = os.cpu_count() or 1
    times = []
    while len(times) < max(1, args.steps):
        t0 = time.perf_counter()
        orc.run(X, **p, threads=cores)
        times.append(time.perf_counter() - t0)
        if sum(times) + times[-1] > args.ref_budget:
            break
    t = float(np.mean(times))
    v = X.shape[0] / t
    res = {"value": v, "unit": "points/s", "cores": cores, "kind": "port",
           "sample": "the full %s workload (%d x %d), one complete run per step, %d step(s) in the %.0f s budget; "
                     "%.2f s per run" % (WORKLOAD, X.shape[0], X.shape[1], len(times), args.ref_budget, t)}
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "points/s", "n_gpus": args.gpus,
            "steps": len(times), "warmup": 0, "ms_per_step": 1000.0 * t,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD, "n": int(X.shape[0]), "d": int(X.shape[1]), **p, "seed": args.seed},
            "cpu_baseline": res, "e2e": {"value": v, "unit": "points/s", "h2d_bytes_per_step": 0,
                                         "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    from gpu_inscy_gb300 import synth
    X = synth.make_plain(args.seed, n=args.n)
    p = dict(synth.PARAMS["plain"])
    if args.impl == "reference":
        run_reference(args, X, p)
        return
    ws, rank, local = dist_env()
    import torch
    from gpu_inscy_gb300 import _lib
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    _lib.load()
    params = _lib.make_params(**p)
    n, d = X.shape
    stream = torch.cuda.Stream()
    Xd = torch.from_numpy(X).cuda()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    def device_step():
        with torch.cuda.stream(stream):
            return _lib.run_device(Xd.data_ptr(), n, d, params, stream.cuda_stream)

    for _ in range(args.warmup):
        subs, labels, stats = device_step()
    torch.cuda.synchronize()
    # ---- timed region (device-resident input)
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    times, stats_all = [], []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        subs, labels, stats = device_step()
        e1.record(stream)
        e1.synchronize()
        times.append(e0.elapsed_time(e1))
        stats_all.append(stats)
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms = float(np.mean(times))
    if ws > 1:
        t = torch.tensor([ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    # ---- end to end through the host-buffer C ABI
    e2e_times, e2e_stats = [], None
    for _ in range(max(1, args.steps)):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        s2, l2, e2e_stats = _lib.run_host(X, params)
        e2e_times.append(time.perf_counter() - t0)
    e2e_ms = 1000.0 * float(np.mean(e2e_times))
    same = s2 == subs and np.array_equal(l2, labels)
    # ---- roofline of the density candidate pass (pass-1 launches)
    st = stats_all[-1]
    peak, peak_kind = measured_peak()
    launches = max(1, st["density_launches_pass1"])
    per_launch_ms = st["ms_density_pass1"] / launches
    per_launch_bytes = st["density_bytes"] / launches
    achieved = per_launch_bytes / (per_launch_ms * 1e-3) / 1e9 if per_launch_ms > 0 else 0.0
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "density_traffic.json")
    if os.path.exists(tpath):
        try:
            traffic = json.load(open(tpath)).get("bytes_per_launch")
        except (OSError, ValueError):
            traffic = None
    roof = {"bound": "hbm", "kernel": "k_neighbours_rows<write> (density candidate pass)", "achieved": achieved,
            "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "peak_source": peak_kind, "traffic": traffic,
            "bytes_per_launch": per_launch_bytes, "ms_per_launch": per_launch_ms}
    # the restrict/merge/prune level kernel: its algorithmic bytes over all
    # levels / its device time per run
    tree_gbs = st["tree_bytes"] / (st["ms_tree"] * 1e-3) / 1e9 if st["ms_tree"] > 0 else 0.0
    roof_tree = {"bound": "hbm", "kernel": "k_tree_level (restrict / merge / prune)", "achieved": tree_gbs,
                 "peak": peak, "unit": "GB/s", "frac": tree_gbs / peak, "peak_source": peak_kind,
                 "bytes_per_run": st["tree_bytes"], "ms_per_run": st["ms_tree"]}
    # ---- labels of the timed run against the oracle's (full-size fixture)
    full = args.seed == 0 and n == 25_000
    parity = {"fixture": "tests/golden/full_plain.json" if full else None,
              "labels_bit_exact_vs_oracle": fixture_check("plain", subs, labels) if full else None,
              "device_and_host_entries_agree": bool(same)}
    line = {"metric": METRIC, "value": ws * n / (ms * 1e-3), "unit": "points/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD, "n": n, "d": d, **p, "seed": args.seed,
                       "l2": "flushed before every step (256 MiB write)", "parallelism": "replicas"},
            "e2e": {"value": ws * n / (e2e_ms * 1e-3), "unit": "points/s", "ms_per_step": e2e_ms,
                    "h2d_bytes_per_step": int(e2e_stats["h2d_bytes"]), "d2h_bytes_per_step": int(e2e_stats["d2h_bytes"])},
            "gpu_launches": int(sum(s["kernel_launches"] for s in stats_all)),
            "roofline": roof, "roofline_tree": roof_tree, "parity": parity, "clocks": clk,
            "breakdown_ms": {k: st[k] for k in ("ms_setup", "ms_density", "ms_density_pass1", "ms_tree",
                                               "ms_cluster", "ms_replay", "ms_replay_prune", "ms_replay_cluster",
                                               "ms_replay_join", "ms_d2h", "ms_expand", "ms_commit_tail",
                                               "ms_total")},
            "run": {k: st[k] for k in ("calls", "regions", "subspaces", "levels", "candidates")},
            "commit_counters": st["replay"],
            "autotune": {"rows_takes": int(st["rows_takes"]), "rows_blocks_per_sm": int(st["rows_blocks_per_sm"]),
                         "note": "row-kernel launch shape measured by the engine's tuner in a warm-up run: "
                                 "work-counter updates per warp, resident blocks per SM"},
            "clustered_subspaces": len(subs)}
    if rank == 0 and not args.no_batched:
        line["batched"] = batched_block(_lib)
    if rank == 0 and not args.no_extra:
        line.update(extra_blocks(_lib))
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(X, p, args.cpu_sample)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
