"""Build libinscy_gb300.so (the CUDA engine + C ABI) in-tree, for sm_103a.

Each .cu translation unit is compiled by its own nvcc process (in parallel),
then linked into gpu_inscy_gb300/libinscy_gb300.so.  Floating point is
compiled without multiply-add contraction and with IEEE division and square
root, because the density tests must round exactly as the reference's
host code does.

build_ext() then compiles the PyTorch binding (csrc/torch_binding.cpp, module
inscy_gb300_ext) against that library, in-tree under _build/ext.
"""
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libinscy_gb300.so")
SOURCES = ["engine.cu", "kernels_setup.cu", "kernels_density.cu", "kernels_tree.cu", "kernels_cluster.cu",
           "noalloc.cu", "mlp.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off", "-fmad=false",
         "-prec-div=true", "-prec-sqrt=true", "-ftz=false", "-Xptxas", "-v"]


def nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def _compile(src, verbose):
    out = os.path.join(OBJ, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc(), *ARCH, *FLAGS, "-I", os.path.join(HERE, "..", "include"), "-c", os.path.join(CSRC, src), "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, r.stdout, r.stderr))
    with open(os.path.join(OBJ, os.path.splitext(src)[0] + ".ptxas.txt"), "w") as f:
        f.write(r.stderr)
    if verbose:
        print(r.stderr, file=sys.stderr)
    return out


def build(verbose=False, force=False):
    os.makedirs(OBJ, exist_ok=True)
    srcs = [os.path.join(CSRC, s) for s in SOURCES]
    hdrs = [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".cuh", ".h"))]
    hdrs.append(os.path.join(HERE, "..", "include", "inscy_gb300.h"))
    if not force and os.path.exists(LIB):
        t = os.path.getmtime(LIB)
        if all(os.path.getmtime(p) < t for p in srcs + hdrs):
            return LIB
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), SOURCES))
    cmd = [nvcc(), *ARCH, "-shared", "-o", LIB, *objs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
    return LIB


EXT_NAME = "inscy_gb300_ext"
EXT_DIR = os.path.join(OBJ, "ext")


def build_ext(verbose=False):
    """Compile (or reuse) the PyTorch binding and return the loaded module.

    The module only binds: run_gpu_4 / run_gpu_5 call the C ABI of
    libinscy_gb300.so, which it links with an rpath to this directory."""
    build()
    from torch.utils import cpp_extension
    os.makedirs(EXT_DIR, exist_ok=True)
    return cpp_extension.load(name=EXT_NAME, sources=[os.path.join(CSRC, "torch_binding.cpp")],
                              extra_cflags=["-O2"], extra_ldflags=["-L" + HERE, "-linscy_gb300", "-Wl,-rpath," + HERE],
                              build_directory=EXT_DIR, with_cuda=True, verbose=verbose)


if __name__ == "__main__":
    t = __import__("time").time()
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv), "%.1fs" % (__import__("time").time() - t))
