"""Drop-in replacement of the GPU entry points of python/inscy.py.

`GPU(...)` and `GPU5(...)` take the reference's arguments (a float32 torch
tensor or numpy array [n, d] in [0, 1], neighborhood_size, F, num_obj,
min_size, r, number_of_cells, rectangular, entropy_order) and return the
reference's `(subspaces, clusterings)` pair: a list of ascending dim lists and
a list of per-point label lists, in the reference's result-map order
(python/inscy.py:189-197 -> inscy_map.cpp:979-1158).  The labels are those of
the reference CPU INSCY (`CPU()`, python/inscy.py:121), bit for bit.

The helpers `normalize`, `clean_up` and `count_number_of_clusters` keep the
reference's behaviour (python/inscy.py:37-107).
"""
import numpy as np

from . import _ext, _lib


def _as_numpy(X):
    try:
        import torch
        if isinstance(X, torch.Tensor):
            return X.detach().to("cpu", torch.float32).contiguous().numpy()
    except ImportError:  # pragma: no cover
        pass
    return np.ascontiguousarray(np.asarray(X, dtype=np.float32))


def _run(X, neighborhood_size, F, num_obj, min_size, r, number_of_cells, rectangular, entropy_order, mode,
         as_numpy):
    if not as_numpy:
        # the reference-facing call: the PyTorch extension's run_gpu_4 /
        # run_gpu_5, whose result is already the reference's pair of lists
        import torch
        Xt = X if isinstance(X, torch.Tensor) else torch.from_numpy(_as_numpy(X))
        ext = _ext.load()
        fn = ext.run_gpu_5 if mode == _lib.MODE_BATCHED else ext.run_gpu_4
        subspaces, clusterings = fn(Xt, neighborhood_size, F, num_obj, min_size, r, number_of_cells,
                                    bool(rectangular), entropy_order)
        return subspaces, clusterings
    p = _lib.make_params(neighborhood_size, F, num_obj, min_size, r, number_of_cells, rectangular, entropy_order)
    try:
        import torch
        if isinstance(X, torch.Tensor) and X.is_cuda:
            if X.dtype != torch.float32 or X.dim() != 2:
                raise ValueError("X must be a float32 [n, d] tensor")
            Xc = X.contiguous()
            stream = torch.cuda.current_stream(Xc.device).cuda_stream
            with torch.cuda.device(Xc.device):
                subs, labels, stats = _lib.run_device(Xc.data_ptr(), Xc.shape[0], Xc.shape[1], p, stream, mode)
            return subs, labels
    except ImportError:  # pragma: no cover
        pass
    subs, labels, stats = _lib.run_host(_as_numpy(X), p, mode)
    return subs, labels


def GPU(X, neighborhood_size, F, num_obj, min_size, r=1., number_of_cells=3, rectangular=False, entropy_order=0,
        as_numpy=False):
    """Plain GPU INSCY (replaces python/inscy.py:189 GPU -> run_gpu_4).

    Returns (subspaces, clusterings) as Python lists like the reference,
    through the PyTorch extension's run_gpu_4; with as_numpy=True, through the
    C ABI directly, the clusterings are a list of int32 arrays (no copy)."""
    return _run(X, neighborhood_size, F, num_obj, min_size, r, number_of_cells, rectangular, entropy_order,
                _lib.MODE_PLAIN, as_numpy)


def GPU5(X, neighborhood_size, F, num_obj, min_size, r=1., number_of_cells=3, rectangular=False, entropy_order=0,
         as_numpy=False):
    """Batched GPU INSCY (replaces python/inscy.py:194 GPU5 -> run_gpu_5)."""
    return _run(X, neighborhood_size, F, num_obj, min_size, r, number_of_cells, rectangular, entropy_order,
                _lib.MODE_BATCHED, as_numpy)


def GPU_batch(Xs, neighborhood_size, F, num_obj, min_size, r=1., number_of_cells=3, rectangular=False,
              entropy_order=0):
    """Many independent datasets; returns one (subspaces, labels) pair per dataset."""
    p = _lib.make_params(neighborhood_size, F, num_obj, min_size, r, number_of_cells, rectangular, entropy_order)
    return [(s, l) for s, l, _ in _lib.run_batch([_as_numpy(x) for x in Xs], p)]


def run_stats(X, neighborhood_size, F, num_obj, min_size, r=1., number_of_cells=3, rectangular=False,
              entropy_order=0, mode=_lib.MODE_PLAIN):
    """Run once and also return the engine's statistics dict."""
    p = _lib.make_params(neighborhood_size, F, num_obj, min_size, r, number_of_cells, rectangular, entropy_order)
    return _lib.run_host(_as_numpy(X), p, mode)


def normalize(x):
    """Min-max scale every column to [0, 1] (python/inscy.py:37-41)."""
    min_x = x.min(0, keepdim=True)[0]
    max_x = x.max(0, keepdim=True)[0]
    return (x - min_x) / (max_x - min_x)


def clean_up(subspaces, clusterings, min_size):
    """Drop clusters smaller than min_size and subspaces left without clusters (python/inscy.py:51-85)."""
    subspaces = np.array(subspaces, dtype=object)
    clusterings = np.array(clusterings)
    keep = np.zeros(len(clusterings), bool)
    for i in range(len(clusterings)):
        labels, counts = np.unique(clusterings[i][clusterings[i] >= 0], return_counts=True)
        for lab, cnt in zip(labels, counts):
            if cnt < min_size:
                clusterings[i][clusterings[i] == lab] = -1
        keep[i] = bool(np.any(counts >= min_size))
    return subspaces[keep], clusterings[keep]


def count_number_of_clusters(subspaces, clusterings):
    """Number of distinct non-negative labels summed over subspaces (python/inscy.py:88-107)."""
    return int(sum(len(np.unique(np.asarray(c)[np.asarray(c) >= 0])) for c in clusterings))
