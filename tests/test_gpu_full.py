"""CUDA path vs the oracle at the timed sizes (full-size fixtures).

The fixtures in tests/golden/full_*.json hold the oracle's output
(oracle/inscy_oracle_fast.cpp, pinned to the reference's own outputs) on the
workloads the bench times: the 25,000 x 15 plain workload, 8 datasets of the
64-dataset batch workload (up to 49,994 points, d up to 20) and, where the
fixture was made, the 100,000 x 25 workload.  Per clustered subspace they
store the sha256 of its int32 labels and its cluster count; the inputs are
regenerated from the seeded generators and checked against the stored input
digest first.  All calls go through the C ABI.
"""
import os

import numpy as np
import pytest

from golden_io import GOLDEN, array_digest, assert_digest, full_fixture
from gpu_inscy_gb300 import _lib, synth

pytestmark = pytest.mark.gpu


def regenerate(e):
    if e["generator"] == "make_batch":
        X = synth.make_batch(e["seed"])[e["index"]]
    elif "n_arg" in e:
        X = getattr(synth, e["generator"])(e["seed"], n=e["n_arg"])
    else:
        X = getattr(synth, e["generator"])(e["seed"])
    assert X.shape == (e["n"], e["d"])
    assert array_digest(X.astype("<f4")) == e["x_sha256"], "the generator no longer reproduces %s" % e["name"]
    return X


def test_plain_workload_full_size_matches_oracle(engine):
    e = full_fixture("plain")["entries"][0]
    X = regenerate(e)
    subs, labels, st = _lib.run_host(X, _lib.make_params(**e["params"]))
    assert_digest(subs, labels, e, e["name"])
    assert len(subs) == len(e["subspaces"]) > 1000
    # the device-pointer entry gives the same result
    import torch
    Xd = torch.from_numpy(X).cuda()
    subs2, labels2, _ = _lib.run_device(Xd.data_ptr(), X.shape[0], X.shape[1], _lib.make_params(**e["params"]))
    assert subs2 == subs and np.array_equal(labels2, labels)


@pytest.mark.parametrize("k", range(8))
def test_batch_workload_datasets_match_oracle(engine, k):
    e = full_fixture("batch")["entries"][k]
    X = regenerate(e)
    subs, labels, _ = _lib.run_host(X, _lib.make_params(**e["params"]))
    assert_digest(subs, labels, e, e["name"])


def test_batched_form_matches_oracle(engine):
    """The batched entry (concurrent lanes, a scheduled order) on the fixture
    datasets, largest first."""
    ents = full_fixture("batch")["entries"]
    Xs = [regenerate(e) for e in ents]
    order = list(np.argsort([-x.shape[0] for x in Xs]))
    outs = _lib.run_batch(Xs, _lib.make_params(**ents[0]["params"]), _lib.MODE_BATCHED, order=order, lanes=4)
    for e, (subs, labels, _) in zip(ents, outs):
        assert_digest(subs, labels, e, e["name"] + " (batched)")


@pytest.mark.skipif(not os.path.exists(os.path.join(GOLDEN, "full_large_d.json")),
                    reason="the 100,000 x 25 fixture was not made")
def test_large_d_workload_matches_oracle(engine):
    e = full_fixture("large_d")["entries"][0]
    X = regenerate(e)
    subs, labels, _ = _lib.run_host(X, _lib.make_params(**e["params"]))
    assert_digest(subs, labels, e, e["name"])


@pytest.mark.skipif(not os.path.exists(os.path.join(GOLDEN, "full_large_d_20k.json")),
                    reason="the 20,000 x 25 fixture was not made")
def test_large_d_generator_at_20000_points_matches_oracle(engine):
    """The 100,000 x 25 workload's generator and parameters (d = 25: 32-slot
    point rows; cells = 5; eps = 0.02) at 20,000 points."""
    e = full_fixture("large_d_20k")["entries"][0]
    X = regenerate(e)
    subs, labels, _ = _lib.run_host(X, _lib.make_params(**e["params"]))
    assert_digest(subs, labels, e, e["name"])


@pytest.mark.skipif(not os.path.exists(os.path.join(GOLDEN, "full_plain_entropy.json")),
                    reason="the entropy-order fixture was not made")
@pytest.mark.parametrize("k", range(2))
def test_plain_workload_entropy_orders_match_oracle(engine, k):
    """The 25,000 x 15 workload with entropy_order 1 and -1: permuted SCY-tree
    and neighbourhood-trie level orders at full size."""
    e = full_fixture("plain_entropy")["entries"][k]
    X = regenerate(e)
    subs, labels, _ = _lib.run_host(X, _lib.make_params(**e["params"]))
    assert_digest(subs, labels, e, e["name"])


@pytest.mark.skipif(not os.path.exists(os.path.join(GOLDEN, "full_rect.json")),
                    reason="the rectangular fixture was not made")
@pytest.mark.parametrize("k", range(2))
def test_rectangular_density_at_full_size_matches_oracle(engine, k):
    """rectangular=True (density by neighbour count, the paper's setting) on the
    25,000 x 15 workload and the 100,000 x 25 generator at 20,000 points."""
    e = full_fixture("rect")["entries"][k]
    X = regenerate(e)
    subs, labels, _ = _lib.run_host(X, _lib.make_params(**e["params"]))
    assert_digest(subs, labels, e, e["name"])


@pytest.mark.skipif(not os.path.exists(os.path.join(GOLDEN, "full_large_d_20k_entropy.json")),
                    reason="the 20,000 x 25 entropy-order fixture was not made")
def test_large_d_generator_entropy_order_matches_oracle(engine):
    """entropy_order 1 on the 100,000 x 25 generator at 20,000 points (d = 25,
    five cells: deep permuted tries, 32-slot rows), plain and batched mode."""
    e = full_fixture("large_d_20k_entropy")["entries"][0]
    X = regenerate(e)
    for mode in (_lib.MODE_PLAIN, _lib.MODE_BATCHED):
        subs, labels, _ = _lib.run_host(X, _lib.make_params(**e["params"]), mode)
        assert_digest(subs, labels, e, e["name"] + " mode %d" % mode)
