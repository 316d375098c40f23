"""The oracle against the reference's own outputs (golden fixtures).

The fixtures were produced by the compiled reference CPU INSCY
(`run_cpu3_weak`, inscy_map.cpp:230-270) through tests/golden/make_golden.py.
"""
import numpy as np
import pytest

import oracle as orc
from golden_io import assert_same, family_cases, small_case


@pytest.mark.parametrize("rect", [0, 1])
def test_small_workload_matches_reference(rect):
    X, p, want = small_case(rect)
    assert X.shape == (1500, 5)
    got = orc.run(X, **p)
    assert_same(got, want, "small rect=%d" % rect)
    assert len(want[0]) > 10


@pytest.mark.parametrize("case", family_cases(), ids=lambda c: "family%d" % c[0])
def test_family_matches_reference(case):
    i, X, p, want = case
    got = orc.run(X, **p)
    assert_same(got, want, "family %d" % i)


def test_thread_count_does_not_change_result():
    X, p, want = small_case(0)
    a = orc.run(X, **p, threads=1)
    b = orc.run(X, **p, threads=5)
    assert_same(a, b, "threads")


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
