"""Regenerate the golden fixtures from the compiled reference CPU INSCY.

Runs the reference's own `run_cpu3_weak` (`inscy_map.cpp:230-270`, the
function behind `python/inscy.py:121 CPU()`) built by
`oracle/build_ref.py`, on seeded inputs, and stores inputs, parameters and
outputs as compressed .npz files next to this script.  Needs the reference
sources (only present where the fixtures are made; their root in the
environment variable INSCY_REFERENCE_ROOT); the tests only read the .npz
files.

Fixtures:
  small_rect{0,1}.npz  the 1,500 x 5 workload (4 clusters in 3-dim subspaces,
                       eps=0.05, cells=4), plain and rectangular density;
  family.npz           48 small seeded inputs (n <= 400, d <= 6) sweeping
                       eps, cells, num_obj, min_size, r, rectangular and
                       entropy_order.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pack(subspaces, clusterings, n):
    dims = np.full((len(subspaces), 64), -1, np.int32)
    for i, s in enumerate(subspaces):
        dims[i, :len(s)] = s
    labels = np.array(clusterings, np.int32).reshape(len(subspaces), n)
    return dims, labels


def family_cases(count=48):
    from gpu_inscy_gb300 import synth
    for s in range(count):
        rng = np.random.default_rng(31337 + s)
        n = int(rng.integers(40, 400))
        d = int(rng.integers(1, 7))
        X = synth.make_random(s, n, d, n_clusters=int(rng.integers(1, 5)), std=float(rng.uniform(0.01, 0.1)))
        yield X, dict(neighborhood_size=float(rng.choice([0.03, 0.05, 0.08, 0.1, 0.15, 0.25])), F=1.0,
                      num_obj=int(rng.integers(1, 6)), min_size=int(rng.integers(1, 16)),
                      r=float(rng.choice([0.7, 1.0, 1.3])), number_of_cells=int(rng.integers(2, 7)),
                      rectangular=bool(rng.integers(0, 2)), entropy_order=int(rng.choice([0, 0, 0, 1, -1])))


def run_ref(ref, X, p):
    import torch
    return ref.run_cpu3_weak(torch.from_numpy(X), p["neighborhood_size"], p["F"], p["num_obj"], p["min_size"],
                             p["r"], p["number_of_cells"], p["rectangular"], p["entropy_order"])


def main():
    import build_ref
    from gpu_inscy_gb300 import synth
    ref = build_ref.load()
    for rect in (0, 1):
        X = synth.make_small(0)
        p = dict(synth.PARAMS["small"], rectangular=bool(rect), entropy_order=0)
        subs, clus = run_ref(ref, X, p)
        dims, labels = pack(subs, clus, X.shape[0])
        np.savez_compressed(os.path.join(HERE, "small_rect%d.npz" % rect), X=X, dims=dims, labels=labels,
                            **{k: np.array(v) for k, v in p.items()})
        print("small rect=%d: %d subspaces" % (rect, len(subs)), flush=True)
    rec = {}
    for i, (X, p) in enumerate(family_cases()):
        subs, clus = run_ref(ref, X, p)
        dims, labels = pack(subs, clus, X.shape[0])
        rec["X%d" % i] = X
        rec["dims%d" % i] = dims
        rec["labels%d" % i] = labels
        rec["params%d" % i] = np.array([p["neighborhood_size"], p["F"], p["num_obj"], p["min_size"], p["r"],
                                        p["number_of_cells"], p["rectangular"], p["entropy_order"]], np.float64)
        print("family %d: n=%d d=%d -> %d subspaces" % (i, X.shape[0], X.shape[1], len(subs)), flush=True)
    rec["count"] = np.array(len([k for k in rec if k.startswith("X")]))
    np.savez_compressed(os.path.join(HERE, "family.npz"), **rec)


if __name__ == "__main__":
    main()
