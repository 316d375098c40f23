"""The C-ABI library: it builds, loads, exports what include/inscy_gb300.h
declares, and rejects bad arguments with an error code (no GPU needed)."""
import ctypes
import os
import re

import numpy as np
import pytest

from gpu_inscy_gb300 import _lib

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "inscy_gb300.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(inscy_[a-z_]+)\s*\(", src)))


def test_header_lists_the_python_exports():
    assert declared_functions() == sorted(_lib.EXPORTS)


def test_library_exports_every_declared_symbol(engine):
    for name in declared_functions():
        assert hasattr(engine, name), name


def test_version(engine):
    assert engine.inscy_version().decode().startswith("inscy_gb300")


def _call(engine, X, **kw):
    p = _lib.make_params(**{**dict(neighborhood_size=0.1, F=1.0, num_obj=2, min_size=4, r=1.0,
                                   number_of_cells=4), **kw})
    h = ctypes.c_void_p()
    X = np.ascontiguousarray(X, np.float32)
    rc = engine.inscy_run(X.ctypes.data if X.size else None, X.shape[0], X.shape[1] if X.ndim == 2 else 0,
                          ctypes.byref(p), 0, ctypes.byref(h))
    return rc, h


@pytest.mark.parametrize("kw,code", [
    (dict(neighborhood_size=0.0), _lib.INSCY_ERR_ARG),
    (dict(number_of_cells=0), _lib.INSCY_ERR_ARG),
    (dict(number_of_cells=300), _lib.INSCY_ERR_LIMIT),
])
def test_bad_parameters_are_rejected(engine, kw, code):
    rc, h = _call(engine, np.random.default_rng(0).random((10, 3)), **kw)
    assert rc == code
    assert engine.inscy_last_error().decode()


def test_too_many_dims(engine):
    rc, _ = _call(engine, np.random.default_rng(0).random((4, 65)))
    assert rc == _lib.INSCY_ERR_LIMIT


def test_values_outside_unit_interval(engine):
    X = np.random.default_rng(0).random((10, 3)).astype(np.float32)
    X[3, 1] = 1.5
    rc, _ = _call(engine, X)
    assert rc == _lib.INSCY_ERR_ARG
    X[3, 1] = np.nan
    rc, _ = _call(engine, X)
    assert rc == _lib.INSCY_ERR_ARG


def test_null_output_pointer(engine):
    p = _lib.make_params(0.1, 1.0, 2, 4, 1.0, 4)
    X = np.zeros((2, 2), np.float32)
    assert engine.inscy_run(X.ctypes.data, 2, 2, ctypes.byref(p), 0, None) == _lib.INSCY_ERR_ARG


def test_result_accessors_tolerate_null(engine):
    assert engine.inscy_result_count(None) == 0
    assert engine.inscy_result_n(None) == 0
    assert engine.inscy_result_subspace(None, 0, None, 0) == -1
    assert engine.inscy_result_labels(None, 0, None) == _lib.INSCY_ERR_ARG
    assert engine.inscy_result_labels_ptr(None, 0) is None
    assert engine.inscy_result_subspaces(None, None, 0, None) == -1
    assert engine.inscy_result_label_blocks(None, None) == -1
    assert engine.inscy_result_label_block(None, 0) is None
    assert engine.inscy_result_label_slots(None, None) == _lib.INSCY_ERR_ARG
    assert engine.inscy_result_stats(None, None) == _lib.INSCY_ERR_ARG
    engine.inscy_result_free(None)


def _batch_args(Xs):
    B = len(Xs)
    vp = ctypes.c_void_p
    return ((vp * B)(*[x.ctypes.data for x in Xs]), (ctypes.c_int64 * B)(*[x.shape[0] for x in Xs]),
            (ctypes.c_int * B)(*[x.shape[1] for x in Xs]), (vp * B)(*([1] * B)))


def test_batch_arguments_are_rejected(engine):
    """The batch entries check their arguments before any CUDA call: lanes
    outside [1, 64], an order that is no permutation, a negative count; every
    output handle is left NULL."""
    p = _lib.make_params(0.1, 1.0, 2, 4, 1.0, 4)
    Xs = [np.random.default_rng(i).random((20, 3)).astype(np.float32) for i in range(2)]
    ip = ctypes.POINTER(ctypes.c_int)
    for order, lanes in ((None, 0), (None, 65), ((0, 0), 2), ((0, 2), 2), ((1, -1), 2)):
        ptrs, ns, ds, outs = _batch_args(Xs)
        ordp = None if order is None else ctypes.cast((ctypes.c_int * 2)(*order), ip)
        rc = engine.inscy_run_batch_scheduled(ptrs, ns, ds, 2, ctypes.byref(p), ordp, lanes, outs)
        assert rc == _lib.INSCY_ERR_ARG, (order, lanes)
        assert engine.inscy_last_error().decode()
        assert list(outs) == [None, None], (order, lanes)
    ptrs, ns, ds, outs = _batch_args(Xs)
    assert engine.inscy_run_batch_scheduled(ptrs, ns, ds, -1, ctypes.byref(p), None, 2, outs) == _lib.INSCY_ERR_ARG
    assert engine.inscy_run_batch(ptrs, ns, ds, -1, ctypes.byref(p), _lib.MODE_PLAIN, outs) == _lib.INSCY_ERR_ARG
    # no datasets: nothing to run, success
    assert engine.inscy_run_batch(ptrs, ns, ds, 0, ctypes.byref(p), _lib.MODE_PLAIN, outs) == _lib.INSCY_OK
    assert engine.inscy_run_batch_scheduled(ptrs, ns, ds, 0, ctypes.byref(p), None, 2, outs) == _lib.INSCY_OK


def test_missing_library_fails_loudly(monkeypatch):
    missing = os.path.join(os.path.dirname(_lib.LIB_PATH), "_build", "no_such_library.so")
    assert not os.path.exists(missing)
    monkeypatch.setattr(_lib, "LIB_PATH", missing)
    monkeypatch.setattr(_lib, "_lib", None)
    with pytest.raises(ImportError):
        _lib.load()


def test_torch_binding_builds_with_the_reference_entry_points():
    """The PyTorch extension (the Python binding of the engine) compiles
    against the library and exports the reference extension's run_gpu_4 /
    run_gpu_5 (inscy_map.cpp:979-1158) with its argument names."""
    pytest.importorskip("torch")
    from gpu_inscy_gb300 import _ext
    ext = _ext.load()
    assert ext.version() == _lib.load().inscy_version().decode()
    for name in ("run_gpu_4", "run_gpu_5"):
        doc = getattr(ext, name).__doc__
        for arg in ("X", "neighborhood_size", "F", "num_obj", "min_size", "r", "number_of_cells", "rectangular",
                    "entropy_order"):
            assert arg + ":" in doc, (name, arg)
