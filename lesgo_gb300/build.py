"""In-tree build of the CUDA library ``liblesgo_gpu.so`` for sm_103a.

The solver template is instantiated once per precision form in its own
translation unit; the units compile in parallel and link into one shared
library."""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
LIB = os.path.join(HERE, "liblesgo_gpu.so")
OBJDIR = os.path.join(HERE, "_build")
SOURCES = [os.path.join(CSRC, f) for f in ("solver.cu", "solver_fp32.cu", "solver_fp64.cu", "solver_dw.cu")]
DEPS = SOURCES + sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC)
                        if f.endswith((".cuh", ".hpp"))) + [os.path.join(ROOT, "include", "lesgo_gpu.h")]

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(d) <= t for d in DEPS if os.path.exists(d))


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile the library if it is missing or older than its sources."""
    if not force and up_to_date():
        return LIB
    os.makedirs(OBJDIR, exist_ok=True)
    tag = "%d" % os.getpid()
    objs, procs = [], []
    for src in SOURCES:
        obj = os.path.join(OBJDIR, os.path.basename(src).replace(".cu", ".%s.o" % tag))
        cmd = [nvcc(), *NVCC_FLAGS, "-I" + os.path.join(ROOT, "include"), "-c", src, "-o", obj]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        procs.append((subprocess.Popen(cmd), cmd))
        objs.append(obj)
    failed = [cmd for p, cmd in procs if p.wait() != 0]
    if failed:
        raise subprocess.CalledProcessError(1, failed[0])
    tmp = LIB + ".tmp" + tag
    link = [nvcc(), *ARCH, "-shared", *objs, "-o", tmp]
    if verbose:
        print(" ".join(link), file=sys.stderr)
    subprocess.run(link, check=True)
    os.replace(tmp, LIB)
    for o in objs:
        os.remove(o)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
