"""The commit's host threads (gpu_inscy_gb300/csrc/host_threads.h) on the CPU.

The header is plain C++17: the task pool of the commit's parallel loops and
the helper that fills label blocks ahead of it are built with g++ and checked
for every task run once, a task's exception reaching the caller only after all
tasks have ended (the pool stays usable), and label blocks of -1 of the
requested size.
"""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
BUILD = os.path.join(ROOT, "gpu_inscy_gb300", "_build")


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_host_pool_and_block_filler():
    os.makedirs(BUILD, exist_ok=True)
    exe = os.path.join(BUILD, "host_threads_check")
    subprocess.run(["g++", "-O1", "-std=c++17", "-pthread", "-I", os.path.join(ROOT, "gpu_inscy_gb300", "csrc"),
                    os.path.join(HERE, "host_threads_check.cpp"), "-o", exe], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip().endswith("ok"), r.stdout + r.stderr
