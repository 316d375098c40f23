"""Generate the real-shape fixtures from the oracle.

Stand-ins with the sizes of the reference's real-data runs (glass, vowel,
pendigits, sky; `gpu_inscy_gb300.synth.REAL_SHAPES`), run with its real-data
parameters (`synth.real_params`, rectangular density).  The oracle is pinned
against the reference's outputs by tests/test_oracle.py.

    python tests/golden/make_real_shapes.py      (about a minute on 8 cores)

real_shapes.npz: cases in the order of REAL_SHAPES, layout of family.npz.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def main():
    import oracle as orc
    from make_golden import pack
    from gpu_inscy_gb300 import synth
    rec = {}
    for i, name in enumerate(synth.REAL_SHAPES):
        X = synth.make_real_shape(name, seed=0)
        p = dict(synth.real_params(X.shape[0]), entropy_order=0)
        subs, labels = orc.run(X, **p)
        dims, lab = pack(subs, labels, X.shape[0])
        rec["X%d" % i] = X
        rec["dims%d" % i] = dims
        rec["labels%d" % i] = lab
        rec["params%d" % i] = np.array([p["neighborhood_size"], p["F"], p["num_obj"], p["min_size"], p["r"],
                                        p["number_of_cells"], p["rectangular"], p["entropy_order"]], np.float64)
        print("%s: n=%d d=%d -> %d subspaces" % (name, X.shape[0], X.shape[1], len(subs)), flush=True)
    rec["count"] = np.array(len(synth.REAL_SHAPES))
    np.savez_compressed(os.path.join(HERE, "real_shapes.npz"), **rec)


if __name__ == "__main__":
    sys.path.insert(0, HERE)
    main()
