"""Build libjqmc_gpu.so in-tree with nvcc for sm_103a (GB300).

    python -m jqmc_gb300.build

The shared object lands in jqmc_gb300/lib/ (git-ignored).  Two translation
units compiled in parallel, one -gencode; about a minute.
"""

from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
SOURCES = [os.path.join(CSRC, "jqmc_gpu.cu"), os.path.join(CSRC, "jqmc_tc.cu")]
HEADERS = [os.path.join(CSRC, "solid_harmonics.cuh"), os.path.join(CSRC, "jqmc_tc.h"), os.path.join(ROOT, "include", "jqmc_gpu.h")]
OUT_DIR = os.path.join(HERE, "lib")
OUT = os.path.join(OUT_DIR, "libjqmc_gpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def build(verbose: bool = False, force: bool = False) -> str:
    """Compile the translation units in parallel (one -gencode for sm_103a) and
    link them into lib/libjqmc_gpu.so; skipped when the library is newer than
    every source and header."""
    os.makedirs(OUT_DIR, exist_ok=True)
    deps = SOURCES + HEADERS
    if not force and os.path.exists(OUT) and all(os.path.getmtime(OUT) >= os.path.getmtime(d) for d in deps):
        return OUT
    tag = f".tmp{os.getpid()}"
    flags = [*ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", os.path.join(ROOT, "include")]
    if verbose:
        flags.insert(0, "-Xptxas=-v")
    objs, procs = [], []
    for src in SOURCES:
        obj = os.path.join(OUT_DIR, os.path.basename(src).replace(".cu", tag + ".o"))
        cmd = [nvcc(), *flags, "-c", "-o", obj, src]
        if verbose:
            print(" ".join(cmd))
        procs.append(subprocess.Popen(cmd))
        objs.append(obj)
    failed = [p.wait() for p in procs]
    if any(failed):
        raise subprocess.CalledProcessError(max(failed), "nvcc")
    tmp = OUT + tag
    subprocess.run([nvcc(), *ARCH, "-shared", "-o", tmp, *objs], check=True)
    for o in objs:
        os.remove(o)
    os.replace(tmp, OUT)
    return OUT


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force=True))
