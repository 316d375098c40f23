"""Build the engine from its CUDA sources for host execution (the simt harness).

The kernel launches `k<<<grid, block, smem, stream>>>(args)` of the engine's
.cu files are rewritten into `simt::launch("k", grid, block, [=] { k(args); })`
and the files compiled as C++ against tests/simt/cuda_runtime.h.  The device
self-test file that names a device symbol is left out (the harness has no
device symbols).  Output: gpu_inscy_gb300/_build/simt<tag>/driver; `defines`
set the engine's build-time tunables.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
CSRC = os.path.join(ROOT, "gpu_inscy_gb300", "csrc")
OUT = os.path.join(ROOT, "gpu_inscy_gb300", "_build", "simt")
SKIP = {"noalloc.cu", "mlp.cu"}  # not on the clustering path (device symbols, named barriers)


def _split_top(s):
    parts, depth, cur = [], 0, ""
    for ch in s:
        if ch in "([{<":
            depth += 1
        elif ch in ")]}>":
            depth -= 1
        if ch == "," and depth == 0:
            parts.append(cur)
            cur = ""
        else:
            cur += ch
    parts.append(cur)
    return [p.strip() for p in parts]


def rewrite_launches(text):
    out, i = [], 0
    while True:
        j = text.find("<<<", i)
        if j < 0:
            out.append(text[i:])
            return "".join(out)
        k, depth = j, 0
        while k > 0:  # the kernel expression, template arguments included
            ch = text[k - 1]
            if ch == ">":
                depth += 1
            elif ch == "<":
                depth -= 1
            elif depth == 0 and not (ch.isalnum() or ch in "_:"):
                break
            k -= 1
        kexpr = text[k:j]
        e = text.find(">>>", j)
        cfg = _split_top(text[j + 3:e])
        p = e + 3
        while text[p].isspace():
            p += 1
        assert text[p] == "(", text[j - 40:p + 40]
        depth, q = 0, p
        while True:
            if text[q] == "(":
                depth += 1
            elif text[q] == ")":
                depth -= 1
                if depth == 0:
                    break
            q += 1
        out.append(text[i:k])
        out.append('::simt::launch("%s", dim3(%s), dim3(%s), [=]() { %s(%s); })'
                   % (kexpr, cfg[0], cfg[1], kexpr, text[p + 1:q]))
        i = q + 1


def build(verbose=False, defines=(), tag=""):
    out = OUT + tag
    src = os.path.join(out, "src")
    if os.path.isdir(src):
        shutil.rmtree(src)
    os.makedirs(src)
    units = []
    for name in sorted(os.listdir(CSRC)):
        if not name.endswith((".cu", ".cuh", ".h")) or name in SKIP:
            continue
        text = rewrite_launches(open(os.path.join(CSRC, name)).read())
        text = text.replace('asm volatile("mov.u32 %0, %%lanemask_lt;" : "=r"(m));',
                            "m = (1u << (threadIdx.x & 31u)) - 1u;")
        text = text.replace('#include "../../include/inscy_gb300.h"', '#include "inscy_gb300.h"')
        dst = os.path.join(src, name[:-3] + ".cpp" if name.endswith(".cu") else name)
        open(dst, "w").write(text)
        if name.endswith(".cu"):
            units.append(dst)
    units += [os.path.join(HERE, "simt.cpp"), os.path.join(HERE, "driver.cpp")]
    # no _FORTIFY_SOURCE: its longjmp check rejects the jumps between fiber stacks
    flags = ["g++", "-std=c++17", "-O2", "-g", "-U_FORTIFY_SOURCE", "-D_FORTIFY_SOURCE=0", "-ffp-contract=off",
             "-fno-strict-aliasing", "-w",
             "-I" + HERE, "-I" + os.path.join(ROOT, "include"), "-I" + src] + ["-D" + x for x in defines]

    def cc(u):
        obj = os.path.join(out, os.path.basename(u) + ".o")
        r = subprocess.run(flags + ["-c", u, "-o", obj], capture_output=True, text=True)
        if r.returncode:
            raise RuntimeError("compiling %s:\n%s" % (u, r.stderr[-4000:]))
        return obj

    with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        objs = list(ex.map(cc, units))
    exe = os.path.join(out, "driver")
    subprocess.run(["g++", "-o", exe] + objs + ["-lpthread"], check=True)
    if verbose:
        print(exe)
    return exe


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
