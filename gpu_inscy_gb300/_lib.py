"""ctypes binding of libinscy_gb300.so (the C ABI declared in include/inscy_gb300.h).

The CUDA library is the product: if it is missing this module raises, there
is no fallback path.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libinscy_gb300.so")

INSCY_OK = 0
INSCY_ERR_ARG = 1
INSCY_ERR_CUDA = 2
INSCY_ERR_UNSUPPORTED = 3
INSCY_ERR_LIMIT = 4
INSCY_ERR_INTERNAL = 5
MODE_PLAIN = 0
MODE_BATCHED = 1

# every symbol include/inscy_gb300.h declares
EXPORTS = ["inscy_run", "inscy_run_device", "inscy_run_batch", "inscy_run_batch_scheduled", "inscy_result_count", "inscy_result_n",
           "inscy_result_subspace", "inscy_result_labels", "inscy_result_labels_ptr", "inscy_result_subspaces",
           "inscy_result_label_blocks", "inscy_result_label_block", "inscy_result_label_slots", "inscy_result_stats",
           "inscy_result_free", "inscy_last_error", "inscy_version", "inscy_selftest", "inscy_selftest_noalloc",
           "inscy_mlp_params", "inscy_mlp_train", "inscy_mlp_predict", "inscy_mlp_grad", "inscy_mlp_last_error"]


class Params(ctypes.Structure):
    _fields_ = [("neighborhood_size", ctypes.c_float), ("F", ctypes.c_float), ("num_obj", ctypes.c_int),
                ("min_size", ctypes.c_int), ("r", ctypes.c_float), ("number_of_cells", ctypes.c_int),
                ("rectangular", ctypes.c_int), ("entropy_order", ctypes.c_int)]


class Stats(ctypes.Structure):
    _fields_ = [(name, ctypes.c_double) for name in
                ("ms_total", "ms_setup", "ms_density", "ms_density_pass1", "ms_tree", "ms_cluster", "ms_replay",
                 "ms_replay_prune", "ms_replay_cluster", "ms_replay_join", "ms_d2h", "density_bytes", "tree_bytes")] + \
               [(name, ctypes.c_longlong) for name in
                ("density_launches_pass1", "kernel_launches", "calls", "regions", "subspaces", "candidates",
                 "levels", "h2d_bytes", "d2h_bytes")] + [("replay_counters", ctypes.c_longlong * 10), ("ms_expand", ctypes.c_double),
                                               ("ms_commit_tail", ctypes.c_double),
                                               ("rows_takes", ctypes.c_int), ("rows_blocks_per_sm", ctypes.c_int),
                                               ("ms_tune", ctypes.c_double)]

    COUNTERS = ("joins", "new_entries", "label_writes", "border_writes", "superset_entries", "redundancy_points",
                "prune_calls", "prune_points", "clusters_numbered", "border_checks")

    def as_dict(self):
        out = {name: getattr(self, name) for name, _ in self._fields_ if name != "replay_counters"}
        out["replay"] = dict(zip(self.COUNTERS, list(self.replay_counters)))
        return out


class InscyError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("inscy error %d: %s" % (code, msg))
        self.code = code


_lib = None


def load():
    """Load the library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError("libinscy_gb300.so not found at %s; build it with "
                          "`python -c 'import __graft_entry__ as g; g.build()'`" % LIB_PATH)
    lib = ctypes.CDLL(LIB_PATH)
    vp, i64, c_int = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int
    lib.inscy_run.argtypes = [vp, i64, c_int, ctypes.POINTER(Params), c_int, ctypes.POINTER(vp)]
    lib.inscy_run_device.argtypes = [vp, i64, c_int, ctypes.POINTER(Params), c_int, vp, ctypes.POINTER(vp)]
    lib.inscy_run_batch.argtypes = [ctypes.POINTER(vp), ctypes.POINTER(i64), ctypes.POINTER(c_int), c_int,
                                    ctypes.POINTER(Params), c_int, ctypes.POINTER(vp)]
    lib.inscy_run_batch_scheduled.argtypes = [ctypes.POINTER(vp), ctypes.POINTER(i64), ctypes.POINTER(c_int), c_int,
                                              ctypes.POINTER(Params), ctypes.POINTER(c_int), c_int,
                                              ctypes.POINTER(vp)]
    fp = ctypes.POINTER(ctypes.c_float)
    lib.inscy_mlp_params.argtypes = [c_int, c_int]
    lib.inscy_mlp_train.argtypes = [fp, c_int, c_int, fp, fp, c_int, c_int, ctypes.c_float, fp]
    lib.inscy_mlp_predict.argtypes = [fp, c_int, c_int, fp, c_int, fp]
    lib.inscy_mlp_grad.argtypes = [fp, c_int, c_int, fp, fp, c_int, fp, fp]
    lib.inscy_mlp_last_error.restype = ctypes.c_char_p
    lib.inscy_result_count.argtypes = [vp]
    lib.inscy_result_n.argtypes = [vp]
    lib.inscy_result_n.restype = i64
    lib.inscy_result_subspace.argtypes = [vp, c_int, vp, c_int]
    lib.inscy_result_labels.argtypes = [vp, c_int, vp]
    lib.inscy_result_labels_ptr.argtypes = [vp, c_int]
    lib.inscy_result_labels_ptr.restype = vp
    lib.inscy_result_subspaces.argtypes = [vp, vp, c_int, vp]
    lib.inscy_result_label_blocks.argtypes = [vp, ctypes.POINTER(c_int)]
    lib.inscy_result_label_block.argtypes = [vp, c_int]
    lib.inscy_result_label_block.restype = vp
    lib.inscy_result_label_slots.argtypes = [vp, vp]
    lib.inscy_selftest.argtypes = [i64]
    lib.inscy_selftest.restype = i64
    lib.inscy_selftest_noalloc.argtypes = [i64, vp]
    lib.inscy_selftest_noalloc.restype = i64
    lib.inscy_result_stats.argtypes = [vp, ctypes.POINTER(Stats)]
    lib.inscy_result_free.argtypes = [vp]
    lib.inscy_result_free.restype = None
    lib.inscy_last_error.restype = ctypes.c_char_p
    lib.inscy_version.restype = ctypes.c_char_p
    _lib = lib
    return lib


def make_params(neighborhood_size, F, num_obj, min_size, r, number_of_cells, rectangular=False, entropy_order=0):
    return Params(float(neighborhood_size), float(F), int(num_obj), int(min_size), float(r), int(number_of_cells),
                  int(bool(rectangular)), int(entropy_order))


def check(rc):
    if rc != INSCY_OK:
        raise InscyError(rc, load().inscy_last_error().decode())


class _Owner:
    """Frees a result handle once no label view refers to it any more."""

    def __init__(self, handle):
        self.handle = handle

    def __del__(self):
        if self.handle and _lib is not None:
            _lib.inscy_result_free(self.handle)
            self.handle = None


class _View:
    """numpy view of a block of label rows inside a result (no copy)."""

    def __init__(self, owner, ptr, rows, n):
        self.owner = owner
        self.__array_interface__ = {"shape": (rows, n), "typestr": "<i4", "data": (ptr, True), "version": 3}


def collect(handle):
    """Turn a result handle into (subspaces: list[list[int]], labels, stats).

    `labels` is a list of int32 arrays of length n, one per clustered
    subspace, viewing the result's memory (freed when the last view dies).
    The result is read in a few calls: all subspaces at once, the label
    blocks as 2-d views, and each subspace's row of them.
    """
    lib = load()
    owner = _Owner(handle)
    k = lib.inscy_result_count(handle)
    n = lib.inscy_result_n(handle)
    subspaces, labels = [], []
    if k > 0:
        lens = np.zeros(k, np.int32)
        flat = np.zeros(64 * k, np.int32)
        w = lib.inscy_result_subspaces(handle, flat.ctypes.data, flat.size, lens.ctypes.data)
        if w < 0:
            raise RuntimeError("inscy_result_subspaces failed")
        fl, o = flat[:w].tolist(), 0
        for m in lens.tolist():
            subspaces.append(fl[o:o + m])
            o += m
        if n:
            rows = ctypes.c_int(0)
            nb = lib.inscy_result_label_blocks(handle, ctypes.byref(rows))
            blocks = [np.asarray(_View(owner, lib.inscy_result_label_block(handle, b), rows.value, n))
                      for b in range(nb)]
            slots = np.zeros(k, np.int32)
            check(lib.inscy_result_label_slots(handle, slots.ctypes.data))
            r = rows.value
            labels = [blocks[s // r][s % r] for s in slots.tolist()]
        else:
            labels = [np.empty(0, np.int32) for _ in range(k)]
    st = Stats()
    check(lib.inscy_result_stats(handle, ctypes.byref(st)))
    return subspaces, labels, st.as_dict()


def run_host(X, params, mode=MODE_PLAIN):
    X = np.ascontiguousarray(X, dtype=np.float32)
    if X.ndim != 2:
        raise ValueError("X must be [n, d]")
    h = ctypes.c_void_p()
    check(load().inscy_run(X.ctypes.data, X.shape[0], X.shape[1], ctypes.byref(params), mode, ctypes.byref(h)))
    return collect(h)


def run_device(ptr, n, d, params, stream=0, mode=MODE_PLAIN):
    h = ctypes.c_void_p()
    check(load().inscy_run_device(ctypes.c_void_p(ptr), n, d, ctypes.byref(params), mode, ctypes.c_void_p(stream),
                                  ctypes.byref(h)))
    return collect(h)


def run_batch(Xs, params, mode=MODE_BATCHED, order=None, lanes=None):
    """Many datasets: mode PLAIN one after another; BATCHED on concurrent lanes,
    taking the datasets in `order` (default 0, 1, ...) over `lanes` lanes
    (default 4).  Returns one (subspaces, labels, stats) per dataset, in input order."""
    Xs = [np.ascontiguousarray(x, dtype=np.float32) for x in Xs]
    B = len(Xs)
    ptrs = (ctypes.c_void_p * B)(*[x.ctypes.data for x in Xs])
    ns = (ctypes.c_int64 * B)(*[x.shape[0] for x in Xs])
    ds = (ctypes.c_int * B)(*[x.shape[1] for x in Xs])
    outs = (ctypes.c_void_p * B)()
    if mode == MODE_BATCHED and (order is not None or lanes is not None):
        ordp = None if order is None else (ctypes.c_int * B)(*[int(i) for i in order])
        check(load().inscy_run_batch_scheduled(ptrs, ns, ds, B, ctypes.byref(params),
                                               ctypes.cast(ordp, ctypes.POINTER(ctypes.c_int)),
                                               int(lanes if lanes is not None else 4), outs))
    else:
        check(load().inscy_run_batch(ptrs, ns, ds, B, ctypes.byref(params), mode, outs))
    return [collect(outs[i]) for i in range(B)]


# ---------------------------------------------------------------- cost model
def _fptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def _mlp_check(rc):
    if rc != 0:
        raise InscyError(rc, load().inscy_mlp_last_error().decode())


def mlp_nparams(n_in, hidden=64):
    return int(load().inscy_mlp_params(n_in, hidden))


def mlp_train(params, X, y, steps, lr):
    """Full-batch Adam on the GPU; returns (new params, loss before each step)."""
    params = np.array(params, dtype=np.float32, copy=True)
    X = np.ascontiguousarray(X, dtype=np.float32)
    y = np.ascontiguousarray(y, dtype=np.float32)
    hist = np.zeros(max(1, steps), np.float32)
    _mlp_check(load().inscy_mlp_train(_fptr(params), X.shape[1], 64, _fptr(X), _fptr(y), X.shape[0], steps, lr,
                                      _fptr(hist)))
    return params, hist[:steps]


def mlp_predict(params, X):
    params = np.ascontiguousarray(params, dtype=np.float32)
    X = np.ascontiguousarray(X, dtype=np.float32)
    out = np.zeros(X.shape[0], np.float32)
    _mlp_check(load().inscy_mlp_predict(_fptr(params), X.shape[1], 64, _fptr(X), X.shape[0], _fptr(out)))
    return out


def mlp_grad(params, X, y):
    """(loss, gradient) of the mean squared error at params, computed on the GPU."""
    params = np.ascontiguousarray(params, dtype=np.float32)
    X = np.ascontiguousarray(X, dtype=np.float32)
    y = np.ascontiguousarray(y, dtype=np.float32)
    grad = np.zeros_like(params)
    loss = np.zeros(1, np.float32)
    _mlp_check(load().inscy_mlp_grad(_fptr(params), X.shape[1], 64, _fptr(X), _fptr(y), X.shape[0], _fptr(grad),
                                     _fptr(loss)))
    return float(loss[0]), grad
