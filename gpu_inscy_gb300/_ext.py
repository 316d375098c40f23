"""The PyTorch extension binding: run_gpu_4 / run_gpu_5 with the arguments and
the [subspaces, clusterings] result of the reference's own extension
(inscy_map.cpp:979-1158), compiled in-tree by build.build_ext() over the C ABI
of libinscy_gb300.so.  Fails loudly when it cannot be built or loaded."""
_mod = None


def load():
    global _mod
    if _mod is None:
        from . import build
        _mod = build.build_ext()
    return _mod
