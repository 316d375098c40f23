"""Python access to the INSCY CPU oracles -- TEST INFRASTRUCTURE ONLY.

`run(X, ...)` executes a C++ restatement of the reference CPU INSCY
(`run_cpu3_weak`, inscy_map.cpp:230-270) and returns the reference's
(subspaces, labels) pair.  Two restatements, both pinned to the reference's
own outputs in tests/golden/:

* impl="fast" (default): oracle/inscy_oracle_fast.cpp, neighbour lists derived
  from the parent call's lists, thread pool -- minutes at 100,000 points;
* impl="trie": oracle/inscy_oracle.cpp, the pointer trie with a candidate
  search per query -- hours beyond a few thousand points; the independent
  cross-check of the fast form.

Only tests/, the fixture scripts in tests/golden/, __graft_entry__.smoke()
and bench.py's CPU leg use it, as the checker.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SOURCES = [os.path.join(HERE, s) for s in ("inscy_oracle.cpp", "inscy_oracle_fast.cpp")]
DEPS = SOURCES + [os.path.join(HERE, "oracle_common.h")]
OUT_DIR = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT_DIR, "libinscy_oracle.so")
# -ffp-contract=off: no fused multiply-add, so x86 and Arm round identically
CXXFLAGS = ["-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-pthread"]

_lib = None


def build(force=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(LIB) and all(os.path.getmtime(LIB) > os.path.getmtime(s) for s in DEPS):
        return LIB
    cmd = ["g++", *CXXFLAGS, "-o", LIB, *SOURCES]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stderr)
    return LIB


def load():
    global _lib
    if _lib is None:
        build()
        lib = ctypes.CDLL(LIB)
        i, f, vp = ctypes.c_int, ctypes.c_float, ctypes.c_void_p
        lib.orc_run.argtypes = [vp, i, i, f, f, i, i, f, i, i, i, i, ctypes.POINTER(vp)]
        lib.orcf_run.argtypes = lib.orc_run.argtypes
        lib.orc_count.argtypes = [vp]
        lib.orc_subspace.argtypes = [vp, i, vp, i]
        lib.orc_labels.argtypes = [vp, i, vp]
        lib.orc_stats.argtypes = [vp, vp]
        lib.orc_free.argtypes = [vp]
        lib.orc_free.restype = None
        for name in ("orc_alpha", "orc_expden"):
            getattr(lib, name).argtypes = [i, f, i]
            getattr(lib, name).restype = f
        lib.orc_omega.argtypes = [i]
        lib.orc_omega.restype = f
        _lib = lib
    return _lib


def run(X, neighborhood_size, F, num_obj, min_size, r=1.0, number_of_cells=3, rectangular=False, entropy_order=0,
        threads=None, with_stats=False, impl="fast"):
    """Reference CPU INSCY on X (float32 [n, d]); returns (subspaces, labels[k, n])."""
    lib = load()
    X = np.ascontiguousarray(X, dtype=np.float32)
    n, d = X.shape
    if threads is None:
        threads = os.cpu_count() or 1
    entry = {"fast": lib.orcf_run, "trie": lib.orc_run}[impl]
    h = ctypes.c_void_p()
    rc = entry(X.ctypes.data, n, d, neighborhood_size, F, num_obj, min_size, r, number_of_cells,
               int(bool(rectangular)), int(entropy_order), int(threads), ctypes.byref(h))
    if rc != 0:
        raise RuntimeError("oracle rejected the arguments (rc=%d)" % rc)
    try:
        k = lib.orc_count(h)
        buf = np.zeros(64, np.int32)
        subs = []
        labels = np.empty((k, n), np.int32)
        for i in range(k):
            m = lib.orc_subspace(h, i, buf.ctypes.data, 64)
            subs.append([int(v) for v in buf[:m]])
            if n:
                lib.orc_labels(h, i, labels[i].ctypes.data)
        stats = np.zeros(6, np.int64)
        lib.orc_stats(h, stats.ctypes.data)
    finally:
        lib.orc_free(h)
    if with_stats:
        names = ("calls", "regions", "prunes_passed", "clusterings", "dense_tests", "result_entries")
        return subs, labels, dict(zip(names, (int(v) for v in stats)))
    return subs, labels
