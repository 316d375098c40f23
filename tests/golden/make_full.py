"""Full-size fixtures: the fast oracle's output on the timed workloads.

The reference CPU INSCY cannot run these sizes (about 10^6 s at 25,000 x 15),
so the oracle restatement in oracle/inscy_oracle_fast.cpp -- pinned to the
reference's own outputs by tests/golden/make_golden.py's fixtures and
cross-checked against the trie restatement -- produces them.  Each fixture
holds, per workload, the generator and seed, a digest of the generated input,
the parameters, and per clustered subspace (in the result map's order) the
sha256 of its int32 label vector and its cluster count.  The tests regenerate
the input, check its digest, run the CUDA path and compare digests.

Usage:  python tests/golden/make_full.py plain batch large_d   (any subset)
  plain    the 25,000 x 15 workload, seed 0           -> full_plain.json
  batch    8 datasets of the 64-dataset batch workload, seed 0, including
           the largest (48,807 x 20)                  -> full_batch.json
  large_d  the 100,000 x 25 workload, seed 0           -> full_large_d.json
  large_d_20k  the same generator and parameters at 20,000 points (d = 25,
           cells = 5, eps = 0.02), seed 0             -> full_large_d_20k.json
  plain_entropy  the 25,000 x 15 workload, seed 0, with entropy_order 1 and
           -1 (permuted level orders)                 -> full_plain_entropy.json
  rect     rectangular density (neighbour counts, the paper's setting): the
           25,000 x 15 workload and the 100,000 x 25 generator at 20,000
           points, seed 0                             -> full_rect.json
  large_d_20k_entropy  the 100,000 x 25 generator at 20,000 points with
           entropy_order 1 (d = 25: 32-slot rows, five cells)
                                                      -> full_large_d_20k_entropy.json
"""
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (ROOT, os.path.join(ROOT, "oracle"), os.path.dirname(HERE)):
    if p not in sys.path:
        sys.path.insert(0, p)

# datasets of synth.make_batch(0) in the batch fixture: the largest by n^2 d
# (48,807 x 20), the largest n (49,994 x 17), and six more across the range
BATCH_PICK = [56, 26, 17, 53, 12, 42, 11, 0]


def entry(name, X, params, **meta):
    import oracle as orc
    from golden_io import array_digest, result_digest
    t = time.time()
    subs, labels, st = orc.run(X, **params, with_stats=True)
    dt = time.time() - t
    e = dict(meta, name=name, n=int(X.shape[0]), d=int(X.shape[1]), x_sha256=array_digest(X.astype("<f4")),
             params=params, oracle_s=round(dt, 1), oracle_stats=st)
    e.update(result_digest(subs, labels))
    print("%s: %d x %d -> %d subspaces in %.1f s" % (name, X.shape[0], X.shape[1], len(subs), dt), flush=True)
    return e


def main(which):
    from gpu_inscy_gb300 import synth
    if "plain" in which:
        X = synth.make_plain(0)
        out = {"workload": "plain_n25000_d15", "entries": [entry("plain_seed0", X, dict(synth.PARAMS["plain"]),
                                                                 generator="make_plain", seed=0)]}
        with open(os.path.join(HERE, "full_plain.json"), "w") as f:
            json.dump(out, f)
    if "batch" in which:
        Xs = synth.make_batch(0)
        ents = [entry("batch_seed0_ds%d" % i, Xs[i], dict(synth.PARAMS["batch"]), generator="make_batch", seed=0,
                      index=i) for i in BATCH_PICK]
        with open(os.path.join(HERE, "full_batch.json"), "w") as f:
            json.dump({"workload": "batch64_seed0", "entries": ents}, f)
    if "plain_entropy" in which:
        X = synth.make_plain(0)
        ents = [entry("plain_seed0_e%d" % eo, X, dict(synth.PARAMS["plain"], entropy_order=eo), generator="make_plain",
                      seed=0) for eo in (1, -1)]
        with open(os.path.join(HERE, "full_plain_entropy.json"), "w") as f:
            json.dump({"workload": "plain_n25000_d15_entropy", "entries": ents}, f)
    if "rect" in which:
        ents = [entry("plain_seed0_rect", synth.make_plain(0), dict(synth.PARAMS["plain"], rectangular=True),
                      generator="make_plain", seed=0),
                entry("large_d_20k_seed0_rect", synth.make_large_d(0, n=20_000),
                      dict(synth.PARAMS["large_d"], rectangular=True), generator="make_large_d", seed=0,
                      n_arg=20_000)]
        with open(os.path.join(HERE, "full_rect.json"), "w") as f:
            json.dump({"workload": "rectangular", "entries": ents}, f)
    if "large_d_20k_entropy" in which:
        X = synth.make_large_d(0, n=20_000)
        out = {"workload": "large_d_n20000_d25_entropy",
               "entries": [entry("large_d_20k_seed0_e1", X, dict(synth.PARAMS["large_d"], entropy_order=1),
                                 generator="make_large_d", seed=0, n_arg=20_000)]}
        with open(os.path.join(HERE, "full_large_d_20k_entropy.json"), "w") as f:
            json.dump(out, f)
    if "large_d_20k" in which:
        X = synth.make_large_d(0, n=20_000)
        out = {"workload": "large_d_n20000_d25", "entries": [entry("large_d_20k_seed0", X, dict(synth.PARAMS["large_d"]),
                                                                   generator="make_large_d", seed=0, n_arg=20_000)]}
        with open(os.path.join(HERE, "full_large_d_20k.json"), "w") as f:
            json.dump(out, f)
    if "large_d" in which:
        X = synth.make_large_d(0)
        out = {"workload": "large_d_n100000_d25", "entries": [entry("large_d_seed0", X, dict(synth.PARAMS["large_d"]),
                                                                    generator="make_large_d", seed=0)]}
        with open(os.path.join(HERE, "full_large_d.json"), "w") as f:
            json.dump(out, f)


if __name__ == "__main__":
    main(set(sys.argv[1:]) or {"plain", "batch"})
