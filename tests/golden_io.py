"""Readers of the golden fixtures made by tests/golden/make_golden.py."""
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
