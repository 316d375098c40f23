"""Generate the wide fixtures (d = 17 .. 40) from the oracle.

The density pass takes point rows of 32 slots when 16 < d <= 32 and the
general kernel above that, and leaf keys grow to 64 and 128 bits; the
reference-run fixtures (make_golden.py) stop at d = 6 and the oracle is too
slow at these widths to run inside the test suite, so its outputs are stored
here once.  The oracle itself is pinned against the reference's outputs by
tests/test_oracle.py on the reference fixtures.

    python tests/golden/make_wide.py      (about six minutes on 8 cores)

wide.npz: cases i = 0 .. count-1 with X{i}, dims{i}, labels{i}, params{i}
in the layout of family.npz.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

# (n, d, seed, neighborhood_size, rectangular, clusters, std, min_size)
CASES = [(400, 20, 1, 0.03, False, 3, 0.015, 10), (500, 18, 3, 0.03, False, 3, 0.015, 10),
         (300, 28, 2, 0.03, False, 3, 0.015, 10), (350, 17, 4, 0.03, True, 3, 0.015, 10),
         (200, 36, 5, 0.02, False, 2, 0.01, 12), (250, 40, 6, 0.02, False, 2, 0.01, 12)]


def wide_cases():
    from gpu_inscy_gb300 import synth
    for n, d, seed, eps, rect, k, std, min_size in CASES:
        X = synth.make_random(seed, n, d, n_clusters=k, std=std, sub_dims=3)
        yield X, dict(neighborhood_size=eps, F=1.0, num_obj=4, min_size=min_size, r=1.0, number_of_cells=4,
                      rectangular=rect, entropy_order=0)


def main():
    import oracle as orc
    from make_golden import pack
    rec = {}
    for i, (X, p) in enumerate(wide_cases()):
        subs, labels = orc.run(X, **p)
        dims, lab = pack(subs, labels, X.shape[0])
        rec["X%d" % i] = X
        rec["dims%d" % i] = dims
        rec["labels%d" % i] = lab
        rec["params%d" % i] = np.array([p["neighborhood_size"], p["F"], p["num_obj"], p["min_size"], p["r"],
                                        p["number_of_cells"], p["rectangular"], p["entropy_order"]], np.float64)
        print("wide %d: n=%d d=%d -> %d subspaces" % (i, X.shape[0], X.shape[1], len(subs)), flush=True)
    rec["count"] = np.array(len(CASES))
    np.savez_compressed(os.path.join(HERE, "wide.npz"), **rec)


if __name__ == "__main__":
    sys.path.insert(0, HERE)
    main()
