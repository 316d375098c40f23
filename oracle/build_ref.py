"""Compile the reference INSCY torch extension from its own sources, in place.

Test infrastructure only.  The reference (mrjakobdk/GPU_INSCY) is compiled
from the source files where they lie, with the source list that
`python/inscy.py:9-33` hands to `torch.utils.cpp_extension.load`, and with
every build output written to `oracle/_ref/` (the reference tree stays
read-only).  Two include paths are added because CUDA 13 moved
`nvToolsExt.h` (included at `inscy_map.cpp:10`) under `nvtx3/` and
`thrust/` under `cccl/`.

Only the host-side entry `run_cpu3_weak` (`inscy_map.cpp:230-270`) of the
built module is ever called: it is the reference CPU INSCY that pins the
oracle restatement through the golden fixtures in `tests/golden/`.

Usage:  python oracle/build_ref.py REFERENCE_ROOT
        (or REFERENCE_ROOT in the environment variable INSCY_REFERENCE_ROOT)
"""
import os
import sys
import time

SOURCES = [
    "inscy_map.cpp",
    "src/utils/TmpMalloc.cu",
    "src/utils/util.cu",
    "src/utils/util_data.cu",
    "src/utils/MergeUtil.cu",
    "src/utils/RestrictUtils.cu",
    "src/structures/ScyTreeNode.cu",
    "src/structures/ScyTreeArray.cu",
    "src/algorithms/clustering/ClusteringCpu.cu",
    "src/algorithms/clustering/ClusteringGpu.cu",
    "src/algorithms/clustering/ClusteringGpuBlocks.cu",
    "src/algorithms/clustering/ClusteringGpuBlocksMem.cu",
    "src/algorithms/clustering/ClusteringGpuStreams.cu",
    "src/algorithms/inscy/InscyCompare.cu",
    "src/algorithms/inscy/InscyNodeCpu.cu",
    "src/algorithms/inscy/InscyCpuGpuMix.cu",
    "src/algorithms/inscy/InscyCpuGpuMixClStream.cu",
    "src/algorithms/inscy/InscyArrayGpu.cu",
    "src/algorithms/inscy/InscyArrayGpuMulti.cu",
    "src/algorithms/inscy/InscyArrayGpuMulti2.cu",
    "src/algorithms/inscy/InscyArrayGpuMulti2ClMulti.cu",
    "src/algorithms/inscy/InscyArrayGpuMulti2ClMultiMem.cu",
    "src/algorithms/inscy/InscyArrayGpuStream.cu",
]

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")


def reference_root(arg=None):
    """The reference's source tree: the argument, else INSCY_REFERENCE_ROOT."""
    root = arg or os.environ.get("INSCY_REFERENCE_ROOT")
    if not root or not os.path.isdir(root):
        raise RuntimeError("the reference's sources are needed: pass their root or set INSCY_REFERENCE_ROOT")
    return root


def load(ref_root=None, verbose=False):
    """Build (or reuse) the reference module and return it."""
    ref_root = reference_root(ref_root)
    from torch.utils.cpp_extension import load as _load
    os.makedirs(OUT, exist_ok=True)
    os.environ.setdefault("TORCH_CUDA_ARCH_LIST", "10.0")
    cuda_inc = "/usr/local/cuda/include"
    return _load(
        name="inscy_ref",
        sources=[os.path.join(ref_root, s) for s in SOURCES],
        extra_include_paths=[os.path.join(cuda_inc, "nvtx3"), os.path.join(cuda_inc, "cccl")],
        build_directory=OUT,
        verbose=verbose,
    )


if __name__ == "__main__":
    root = reference_root(sys.argv[1] if len(sys.argv) > 1 else None)
    t0 = time.time()
    load(root, verbose=True)
    print("reference module built in %.1f s -> %s" % (time.time() - t0, OUT))
