"""Learned schedule for the batched form (inscy_run_batch_scheduled).

A batch of datasets runs on a few concurrent lanes; each lane takes the next
dataset of the schedule.  With very uneven datasets the makespan depends on
the order: the longest datasets should start first (LPT), which needs their
cost before running them.  This module predicts that cost with a small MLP
(in -> 64 -> 64 -> 1, trained and evaluated by the library's CUDA kernels)
from cheap per-dataset features, trained on cost records logged from the
plain form's own runs.  The schedule only orders work: labels are those of
the plain runs whatever it predicts, and FIFO (the given order) is both its
fallback and the baseline it is judged against (`simulate_makespan`).

Records: `collect_records` runs datasets through the plain entry point and
logs (features, ms per run).  The committed `data/cost_records.json` holds
records measured on a GB300 from the plain runs of the small, plain and batch
workloads (see `collect` at the bottom for the command).
"""
import json
import math
import os
import time

import numpy as np

from . import _lib

HERE = os.path.dirname(os.path.abspath(__file__))
RECORDS = os.path.join(HERE, "data", "cost_records.json")

FEATURES = ("log_n", "d", "log_n_x_d", "cell_max_frac", "cell_entropy", "log_level1_pairs", "sconn_frac",
            "fine_max_frac", "log_eps", "cells", "log_min_size", "num_obj")


def features(X, neighborhood_size, number_of_cells, min_size, num_obj, **_):
    """Per-dataset features: size, dims, and how concentrated the points are on
    the SCY-tree grid and the neighbourhood grid (which drives how far the
    subspace lattice grows and how long the neighbour lists get)."""
    X = np.asarray(X, np.float32)
    n, d = X.shape
    cells = int(number_of_cells)
    eps = float(neighborhood_size)
    G = int(math.ceil(1.0 / eps))
    csz = np.float32(1.0) / np.float32(cells)
    cc = np.minimum((X / csz).astype(np.int64), cells - 1)
    fc = np.minimum((X / (np.float32(1.0) / np.float32(G))).astype(np.int64), G - 1)
    cmax, cent, fmax, pairs = [], [], [], 0.0
    for k in range(d):
        h = np.bincount(cc[:, k], minlength=cells) / max(n, 1)
        cmax.append(h.max())
        nz = h[h > 0]
        cent.append(float(-(nz * np.log(nz)).sum() / math.log(cells)) if cells > 1 else 0.0)
        f = np.bincount(fc[:, k], minlength=G).astype(np.float64)
        fmax.append(f.max() / max(n, 1))
        nb = f + np.concatenate([[0.0], f[:-1]]) + np.concatenate([f[1:], [0.0]])
        pairs += float((f * nb).sum())
    edge = (cc + 1).astype(np.float32) * csz - np.float32(eps)
    sconn = float((X >= edge).mean()) if n else 0.0
    log_n = math.log(max(n, 1))
    return np.array([log_n, d, log_n * d / 20.0, np.mean(cmax), np.mean(cent), math.log(1.0 + pairs / max(n, 1)),
                     sconn, np.mean(fmax), math.log(eps), cells, math.log(max(min_size, 1)), num_obj], np.float32)


def collect_records(datasets, params, repeats=2):
    """Run each (X, params) through the plain entry point; log (features, ms)
    with the time of the fastest of `repeats` runs (the first run warms up)."""
    out = []
    for X, p in zip(datasets, params if isinstance(params, list) else [params] * len(datasets)):
        prm = _lib.make_params(**p)
        best = float("inf")
        for _ in range(repeats):
            t0 = time.perf_counter()
            _lib.run_host(X, prm)
            best = min(best, time.perf_counter() - t0)
        out.append({"features": features(X, **p).tolist(), "ms": 1000.0 * best, "n": int(X.shape[0]),
                    "d": int(X.shape[1])})
    return out


def load_records(path=RECORDS):
    with open(path) as f:
        return json.load(f)["records"]


class CostModel:
    """log(ms) of a plain run from `features`, by the library's MLP kernels."""

    def __init__(self, seed=0):
        self.seed = seed
        self.params = None
        self.mu = self.sd = None
        self.loss_hist = None

    def init_params(self, n_in):
        rng = np.random.default_rng(self.seed)
        H = 64
        W1 = rng.normal(0.0, math.sqrt(2.0 / n_in), (H, n_in))
        W2 = rng.normal(0.0, math.sqrt(2.0 / H), (H, H))
        w3 = rng.normal(0.0, math.sqrt(1.0 / H), H)
        return np.concatenate([W1.ravel(), np.zeros(H), W2.ravel(), np.zeros(H), w3, np.zeros(1)]).astype(np.float32)

    def fit(self, F, ms, steps=3000, lr=3e-3):
        F = np.asarray(F, np.float32)
        self.mu = F.mean(0)
        self.sd = F.std(0) + 1e-6
        y = np.log(np.asarray(ms, np.float64)).astype(np.float32)
        p0 = self.init_params(F.shape[1])
        assert p0.size == _lib.mlp_nparams(F.shape[1])
        self.params, self.loss_hist = _lib.mlp_train(p0, (F - self.mu) / self.sd, y, steps, lr)
        return self

    def predict_log_ms(self, F):
        F = np.asarray(F, np.float32)
        return _lib.mlp_predict(self.params, (F - self.mu) / self.sd)

    def predict_ms(self, F):
        return np.exp(self.predict_log_ms(F))


def lpt_order(costs):
    """Longest (predicted) first: the order the lanes take the datasets in."""
    return [int(i) for i in np.argsort(-np.asarray(costs, np.float64), kind="stable")]


def simulate_makespan(costs, order, lanes):
    """Finish time of `lanes` lanes taking datasets in `order` (true costs)."""
    free = [0.0] * lanes
    for i in order:
        k = int(np.argmin(free))
        free[k] += float(costs[i])
    return max(free) if free else 0.0


def collect(out=RECORDS):
    """Cost records from the plain runs of the small, plain and batch workloads
    (run on a GPU): python -m gpu_inscy_gb300.scheduler"""
    from . import synth
    data, prm = [], []
    for s in range(16):
        data.append(synth.make_small(s))
        prm.append(dict(synth.PARAMS["small"]))
    for s in range(4):
        data.append(synth.make_plain(s, n=[6000, 12000, 25000, 18000][s]))
        prm.append(dict(synth.PARAMS["plain"]))
    for seed in (1, 2, 3):  # seed 0 is the held-out evaluation batch
        for X in synth.make_batch(seed):
            data.append(X)
            prm.append(dict(synth.PARAMS["batch"]))
    _lib.load()
    recs = collect_records(data[:2], prm[:2], repeats=1)  # warm-up
    recs = collect_records(data, prm)
    os.makedirs(os.path.dirname(out), exist_ok=True)
    with open(out, "w") as f:
        json.dump({"features": list(FEATURES), "records": recs}, f)
    return recs


if __name__ == "__main__":
    r = collect(os.environ.get("INSCY_COST_RECORDS", RECORDS))
    print("%d records" % len(r))
