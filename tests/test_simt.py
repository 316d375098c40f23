"""The engine's CUDA sources executed on the host (tests/simt), checked
against the reference outputs -- a CPU check of the kernels themselves.

Every device allocation sits against a guard page, so an out-of-range or
stale index in any kernel faults here; warp collectives must see all 32 lanes
at the same call; and each case runs twice, with the warps of every block in
ascending and in descending order, so a value one warp reads before another
warp has written it without a barrier changes the result.
"""
import os
import shutil
import subprocess
import sys

import numpy as np
import pytest

from golden_io import assert_same, family_cases, real_shape_cases, small_case, wide_cases
from gpu_inscy_gb300 import synth
import oracle as orc

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "simt"))

pytestmark = pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")


@pytest.fixture(scope="module")
def driver():
    import build_simt
    return build_simt.build()


def simt_run(driver, X, p, reverse, tag):
    out_dir = os.path.dirname(driver)
    fx, fo = os.path.join(out_dir, tag + ".f32"), os.path.join(out_dir, tag + ".out")
    X = np.ascontiguousarray(X, np.float32)
    X.tofile(fx)
    n, d = X.shape
    args = [driver, fx, str(n), str(d), repr(float(p["neighborhood_size"])), repr(float(p["F"])), str(p["num_obj"]),
            str(p["min_size"]), repr(float(p["r"])), str(p["number_of_cells"]), str(int(p.get("rectangular", 0))), fo,
            str(int(p.get("entropy_order", 0)))]
    env = dict(os.environ)
    env.pop("SIMT_REVERSE", None)
    if reverse:
        env["SIMT_REVERSE"] = "1"
    r = subprocess.run(args, capture_output=True, text=True, env=env, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    raw = np.fromfile(fo, np.int32)
    k, pos, subs, labs = raw[0], 1, [], []
    for _ in range(k):
        m = raw[pos]
        subs.append(raw[pos + 1:pos + 1 + m].tolist())
        pos += 1 + m
        labs.append(raw[pos:pos + n])
        pos += n
    return subs, (np.stack(labs) if labs else np.zeros((0, n), np.int32))


@pytest.mark.parametrize("reverse", [False, True], ids=["warps-up", "warps-down"])
@pytest.mark.parametrize("rect", [0, 1])
def test_small_workload(driver, rect, reverse):
    X, p, want = small_case(rect)
    assert_same(simt_run(driver, X, p, reverse, "small%d" % rect), want, "small rect=%d" % rect)


def test_family_cases(driver):
    cases = [c for c in family_cases() if c[2]["entropy_order"] == 0][:12]
    for i, X, p, want in cases:
        assert_same(simt_run(driver, X, p, i % 2 == 1, "family%d" % i), want, "family %d" % i)


def test_family_cases_entropy_order(driver):
    # permuted level orders: phantom nodes, cut chains, the neighbourhood
    # walk's partial fine-cell tests
    cases = [c for c in family_cases() if c[2]["entropy_order"] != 0]
    assert cases
    for i, X, p, want in cases:
        assert_same(simt_run(driver, X, p, i % 2 == 1, "family_e%d" % i), want,
                    "family %d (entropy_order %d)" % (i, p["entropy_order"]))


def many_cell_cases():
    """14 cells: with eps above the cell width every point is s-connected on every
    dim and a run merges all 14 cells (the level kernel's radix passes); with a
    smaller eps runs merge a few cells (its partition + merge)."""
    cases = []
    for seed in range(4):
        rng = np.random.default_rng(9100 + seed)
        X = np.clip(rng.normal(0.5, 0.18, (600, 4)), 0, 1).astype(np.float32)
        p = dict(neighborhood_size=[0.09, 0.04][seed % 2], F=0.5, num_obj=2, min_size=6, r=1.0, number_of_cells=14,
                 rectangular=bool(seed // 2), entropy_order=[0, 1, -1, 0][seed])
        cases.append((seed, X, p))
    return cases


def test_many_cells_long_merges(driver):
    for seed, X, p in many_cell_cases():
        assert_same(simt_run(driver, X, p, seed % 2 == 1, "cells%d" % seed), orc.run(X, **p), "14 cells, seed %d" % seed)


def long_list_cases():
    """Two tight clusters of 200 points and 100 noise points in [0, 1]^4, eps
    0.12 / 0.15: every clustered point has ~200 neighbours, so the border walk
    takes a full step of four 32-entry chunks and a partial one, and the union
    walk (the cluster outside the sampled dominant component) several steps of
    two chunks; the noise points near the clusters are border points.  A
    skipped border chunk changes the labels of both cases; the union walk's
    reads are checked against the guard pages here (a tight cluster stays
    connected without a third of its edges), its edges by the bridge cases of
    the build without the link step (below)."""
    cases = []
    for seed, eps in ((1, 0.12), (2, 0.15)):
        rng = np.random.default_rng(seed)
        c1 = rng.normal([0.25, 0.3, 0.7, 0.5], 0.03, (200, 4))
        c2 = rng.normal([0.75, 0.7, 0.3, 0.5], 0.03, (200, 4))
        X = np.clip(np.vstack([c1, c2, rng.uniform(0, 1, (100, 4))]), 0, 1).astype(np.float32)
        p = dict(neighborhood_size=eps, F=1.0, num_obj=4, min_size=20, r=1.0, number_of_cells=3)
        cases.append((seed, X, p))
    return cases


def test_long_neighbour_lists(driver):
    for seed, X, p in long_list_cases():
        want = orc.run(X, **p)
        assert any(len(set(lab.tolist()) - {-1, -2}) >= 2 and (lab == -2).any() for lab in want[1])
        assert_same(simt_run(driver, X, p, seed % 2 == 0, "long%d" % seed), want, "long lists, seed %d" % seed)


def test_wide_rows(driver):
    # d = 20: the density pass on 32-slot point rows; d = 36: the general
    # density kernel and 128-bit leaf keys
    for i, X, p, want in (wide_cases()[0], wide_cases()[4]):
        assert_same(simt_run(driver, X, p, True, "wide%d" % i), want, "wide %d (d=%d)" % (i, X.shape[1]))


def test_real_shapes_small(driver):
    # glass and vowel shapes, real-data parameters (rectangular density)
    for i, X, p, want in real_shape_cases()[:2]:
        assert_same(simt_run(driver, X, p, i % 2 == 1, "real%d" % i), want, "real shape %d" % i)


@pytest.fixture(scope="module")
def driver_big_blocks():
    # every level-kernel work item above 64 points takes the 1024-thread path,
    # every level sizes its neighbour lists with a count pass, and the leaf
    # keys are 128 bits wide
    import build_simt
    return build_simt.build(defines=("INSCY_TREE_BIG=64", "INSCY_SINGLE_PASS_BYTES=0", "INSCY_TREE_MIN_KEY_BYTES=16"),
                            tag="_variant")


@pytest.fixture(scope="module")
def driver_key64():
    import build_simt
    # also keeps the general density kernel (no point rows) for d <= 16
    return build_simt.build(defines=("INSCY_TREE_MIN_KEY_BYTES=8", "INSCY_DENSITY_ROWS=0"), tag="_key64")


@pytest.fixture(scope="module")
def driver_links0():
    import build_simt
    # no link step before the dominant-component sample: the union walk takes
    # every edge (but the sampled point's), so its chunks all count
    return build_simt.build(defines=("INSCY_UF_LINKS=0",), tag="_links0")


def bridge_cases():
    """A small blob (60 points, the lowest point ids) beside a large one (300
    points) and 40 noise points in [0, 1]^3: in subspace {0, 1} the two blobs
    are one cluster, joined by the few pairs that lie within eps across the
    gap.  Without the link step such an edge is taken only from the large
    blob's side (the larger keep index), where the small blob's points come
    after the large blob's neighbours in the list (fine-cell order on dim 0):
    a union walk that drops a list's entries after the first 64, or one chunk
    in three, splits the cluster in each of these cases."""
    cases = []
    for seed, eps, gap in ((0, 0.045, 0.10), (0, 0.05, 0.11), (1, 0.05, 0.12), (3, 0.05, 0.12)):
        rng = np.random.default_rng(seed)
        small = np.column_stack([rng.normal(0.40 + gap, 0.01, 60), rng.normal(0.5, 0.03, 60),
                                 rng.normal(0.5, 0.02, 60)])
        large = np.column_stack([rng.normal(0.40, 0.015, 300), rng.normal(0.5, 0.03, 300),
                                 rng.normal(0.5, 0.02, 300)])
        X = np.clip(np.vstack([small, large, rng.uniform(0, 1, (40, 3))]), 0, 1).astype(np.float32)
        p = dict(neighborhood_size=eps, F=1.0, num_obj=4, min_size=20, r=1.0, number_of_cells=3)
        cases.append((seed, X, p))
    return cases


def test_union_walk_takes_every_edge(driver_links0):
    cases = [(seed, X, p) for seed, X, p in long_list_cases()]
    for _, X, p in bridge_cases():
        subs, labs = orc.run(X, **p)
        lab = labs[subs.index([0, 1])]
        assert lab[0] >= 0 and set(lab[:60].tolist()) == {lab[0]} and lab[60 + int(np.argmax(lab[60:360] >= 0))] == lab[0]
    cases += [(200 + i, X, p) for i, (_, X, p) in enumerate(bridge_cases())]
    cases += [(100 + i, X, p) for i, X, p, _ in [c for c in family_cases() if c[2]["entropy_order"] == 0][:4]]
    for seed, X, p in cases:
        assert_same(simt_run(driver_links0, X, p, seed % 2 == 1, "links0_%d" % seed), orc.run(X, **p),
                    "no link step, case %d" % seed)


@pytest.fixture(scope="module")
def plain_case():
    # the 25,000 x 15 workload's generator and parameters at a size the oracle finishes fast
    X = synth.make_plain(3, n=1000)
    p = dict(synth.PARAMS["plain"])
    return X, p, orc.run(X, **p)


@pytest.mark.parametrize("reverse", [False, True], ids=["warps-up", "warps-down"])
def test_plain_workload_shape(driver, plain_case, reverse):
    X, p, want = plain_case
    assert_same(simt_run(driver, X, p, reverse, "plain"), want, "plain n=1000")


@pytest.mark.parametrize("reverse", [False, True], ids=["warps-up", "warps-down"])
def test_large_blocks_two_pass_lists_wide_keys(driver_big_blocks, plain_case, reverse):
    X, p, want = plain_case
    assert_same(simt_run(driver_big_blocks, X, p, reverse, "plain_big"), want, "plain n=1000, 1024-thread items")
    X, p, want = small_case(0)
    assert_same(simt_run(driver_big_blocks, X, p, reverse, "small_big"), want, "small, 1024-thread items")


def test_64_bit_leaf_keys_general_density_kernel(driver_key64, plain_case):
    X, p, want = plain_case
    assert_same(simt_run(driver_key64, X, p, True, "plain_key64"), want, "plain n=1000, 64-bit keys, no rows")
