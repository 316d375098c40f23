"""The exact (integer) phi step of the density kernel, checked on the host.

phi (ClusteringCpu.cu:118-120) accumulates float(double(sum) + (1 - sq)); the
device computes that step on 64-bit integers (phi_exact.cuh).  The
header compiles as plain C++, so the same code is checked here bit for bit
against the double expression on 20M pseudo-random and edge inputs.
"""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(os.path.dirname(HERE), "gpu_inscy_gb300", "_build")


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_phi_step_exact_matches_double():
    os.makedirs(BUILD, exist_ok=True)
    exe = os.path.join(BUILD, "phi_host_check")
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", os.path.join(HERE, "phi_host_check.cpp"),
                    "-o", exe], check=True)
    out = subprocess.run([exe, "20000000"], check=True, capture_output=True, text=True).stdout.split()
    cases, bad, large = map(int, out[-3:])
    assert cases > 20_000_000
    assert bad == 0, " ".join(out)
    assert large > cases // 10  # sums >= 2^10 (the sticky-bit branch) are exercised
