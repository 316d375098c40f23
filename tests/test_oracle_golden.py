"""The oracles against the reference's own outputs (golden fixtures).

The fixtures were produced by the compiled reference CPU INSCY
(`run_cpu3_weak`, inscy_map.cpp:230-270) through tests/golden/make_golden.py.
Both restatements are checked: the pointer trie ("trie") and the fast form
that derives neighbour lists from the parent call's ("fast"), which also
makes the full-size fixtures.
"""
import numpy as np
import pytest

import oracle as orc
from golden_io import assert_same, family_cases, small_case, wide_cases
from gpu_inscy_gb300 import synth

IMPLS = ["fast", "trie"]


@pytest.mark.parametrize("impl", IMPLS)
@pytest.mark.parametrize("rect", [0, 1])
def test_small_workload_matches_reference(rect, impl):
    X, p, want = small_case(rect)
    assert X.shape == (1500, 5)
    got = orc.run(X, **p, impl=impl)
    assert_same(got, want, "small rect=%d" % rect)
    assert len(want[0]) > 10


@pytest.mark.parametrize("impl", IMPLS)
@pytest.mark.parametrize("case", family_cases(), ids=lambda c: "family%d" % c[0])
def test_family_matches_reference(case, impl):
    i, X, p, want = case
    got = orc.run(X, **p, impl=impl)
    assert_same(got, want, "family %d" % i)


@pytest.mark.parametrize("impl", IMPLS)
def test_thread_count_does_not_change_result(impl):
    X, p, want = small_case(0)
    a = orc.run(X, **p, threads=1, impl=impl)
    b = orc.run(X, **p, threads=5, impl=impl)
    assert_same(a, b, "threads")


def test_fast_oracle_matches_wide_fixtures():
    # d = 17 .. 40, made by the trie oracle (tests/golden/make_wide.py)
    for i, X, p, want in wide_cases():
        assert_same(orc.run(X, **p, impl="fast"), want, "wide %d" % i)


@pytest.mark.parametrize("seed", range(6))
def test_fast_and_trie_oracles_agree(seed):
    """Random inputs beyond the golden family: more points, more dims, eps
    with many s-connections, both density modes and all three dim orders."""
    rng = np.random.default_rng(900 + seed)
    n, d = int(rng.integers(300, 900)), int(rng.integers(3, 8))
    X = synth.make_random(seed + 77, n, d, n_clusters=int(rng.integers(1, 4)), std=float(rng.uniform(0.02, 0.08)))
    p = dict(neighborhood_size=float(rng.choice([0.05, 0.08, 0.12])), F=1.0, num_obj=int(rng.integers(1, 5)),
             min_size=int(rng.integers(2, 12)), r=float(rng.choice([0.8, 1.0])), number_of_cells=int(rng.integers(2, 6)),
             rectangular=bool(seed % 2), entropy_order=[0, 1, -1][seed % 3])
    assert_same(orc.run(X, **p, impl="fast"), orc.run(X, **p, impl="trie"), "seed %d" % seed)


def test_fast_and_trie_oracles_agree_on_plain_generator():
    # the 25,000 x 15 workload's generator and parameters at 2,000 x 15
    X = synth.make_plain(3, n=2000)
    p = synth.PARAMS["plain"]
    assert_same(orc.run(X, **p, impl="fast"), orc.run(X, **p, impl="trie"), "plain 2000")


def test_thresholds_follow_reference_formulas():
    # alpha(d) = 2 n eps^d c(d) / (d + 2), c(d) = 3.14^(d/2) / gamma(d + 2)
    # (ClusteringCpu.cu:145-157), gamma(1)=sqrt(3.14), gamma(2)=1
    lib = orc.load()
    assert lib.orc_omega(3) == np.float32(2.0 / 5.0)
    c1 = np.float32(np.float32(3.14 ** 0.5) / np.float32(np.sqrt(3.14) * 0.5))  # gamma(3) = 0.5*gamma(1)
    a1 = np.float32(np.float32(2 * 1000 * 0.05 * float(c1)) / 3.0)
    assert abs(lib.orc_alpha(1, 0.05, 1000) - a1) <= 1e-4 * a1


def test_empty_input():
    subs, labels = orc.run(np.zeros((0, 3), np.float32), 0.1, 1.0, 2, 4, 1.0, 3)
    assert subs == [] and labels.shape == (0, 0)
