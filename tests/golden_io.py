"""Readers of the golden fixtures made by the scripts in tests/golden/."""
import hashlib
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
PARAM_NAMES = ("neighborhood_size", "F", "num_obj", "min_size", "r", "number_of_cells", "rectangular",
               "entropy_order")


def unpack(dims, labels):
    subs = [[int(v) for v in row if v >= 0] for row in dims]
    return subs, np.asarray(labels, np.int32)


def small_case(rect):
    z = np.load(os.path.join(GOLDEN, "small_rect%d.npz" % rect))
    p = {k: z[k].item() for k in PARAM_NAMES}
    p["num_obj"], p["min_size"], p["number_of_cells"], p["entropy_order"] = (
        int(p["num_obj"]), int(p["min_size"]), int(p["number_of_cells"]), int(p["entropy_order"]))
    p["rectangular"] = bool(p["rectangular"])
    return z["X"], p, unpack(z["dims"], z["labels"])


def family_cases(name="family.npz"):
    z = np.load(os.path.join(GOLDEN, name))
    out = []
    for i in range(int(z["count"])):
        v = z["params%d" % i]
        p = dict(neighborhood_size=float(np.float32(v[0])), F=float(v[1]), num_obj=int(v[2]), min_size=int(v[3]),
                 r=float(np.float32(v[4])), number_of_cells=int(v[5]), rectangular=bool(v[6]),
                 entropy_order=int(v[7]))
        out.append((i, z["X%d" % i], p, unpack(z["dims%d" % i], z["labels%d" % i])))
    return out


def wide_cases():
    """d = 17 .. 40 (32-slot point rows; the general density kernel and 128-bit
    leaf keys above d = 32), made by tests/golden/make_wide.py."""
    return family_cases("wide.npz")


def real_shape_cases():
    """glass, vowel, pendigits, sky shapes with the real-data parameters,
    made by tests/golden/make_real_shapes.py."""
    return family_cases("real_shapes.npz")


def assert_same(got, want, what=""):
    gs, gl = got
    ws, wl = want
    assert [list(s) for s in gs] == [list(s) for s in ws], "%s: subspaces differ\n got %s\nwant %s" % (what, gs, ws)
    if not ws:
        return
    gl = np.asarray(gl, np.int32).reshape(len(gs), -1)
    wl = np.asarray(wl, np.int32).reshape(len(ws), -1)
    for i, s in enumerate(ws):
        bad = np.flatnonzero(gl[i] != wl[i])
        assert bad.size == 0, "%s: labels of subspace %s differ at %d points (first %s: got %d want %d)" % (
            what, s, bad.size, bad[0], gl[i][bad[0]], wl[i][bad[0]])


# --------------------------------------------------------------------------
# Full-size fixtures (tests/golden/make_full.py): the oracle's output on the
# timed workloads, stored as per-subspace digests of the label vectors.
# --------------------------------------------------------------------------
def array_digest(a):
    """sha256 of an array's bytes (little-endian int32 / float32 as stored)."""
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def clusters_of(labels):
    """Number of distinct cluster labels (>= 0), as count_number_of_clusters
    counts them per subspace (python/inscy.py:88-107)."""
    v = np.unique(np.asarray(labels))
    return int((v >= 0).sum())


def result_digest(subs, labels):
    """labels: an int32 array [k, n] or a list of k int32 vectors."""
    rows = [np.asarray(labels[i]).astype("<i4", copy=False) for i in range(len(subs))]
    return {"subspaces": [list(map(int, s)) for s in subs],
            "label_sha256": [array_digest(r) for r in rows],
            "clusters": [clusters_of(r) for r in rows]}


def full_fixture(name):
    with open(os.path.join(GOLDEN, "full_%s.json" % name)) as f:
        return json.load(f)


def assert_digest(got_subs, got_labels, want, what=""):
    """The CUDA path's result against a full-size fixture entry."""
    g = result_digest(got_subs, got_labels)
    assert g["subspaces"] == want["subspaces"], "%s: subspace lists differ (%d vs %d entries)" % (
        what, len(g["subspaces"]), len(want["subspaces"]))
    bad = [i for i, (a, b) in enumerate(zip(g["label_sha256"], want["label_sha256"])) if a != b]
    assert not bad, "%s: labels of %d subspaces differ, first %s" % (what, len(bad), want["subspaces"][bad[0]])
    assert g["clusters"] == want["clusters"]
