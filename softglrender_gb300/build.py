"""Build recipe of the sm_103a renderer library: every .cu under csrc/ is compiled in parallel by
nvcc for sm_103a (one -gencode, --fmad=false, see csrc/sglc_device.cuh) and linked into
softglrender_gb300/_build/libsoftgl_cuda.so (in-tree, git-ignored)."""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
LIB = os.path.join(OUT, "libsoftgl_cuda.so")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"
FLAGS = [ARCH, "-O3", "-lineinfo", "--fmad=false", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler",
         "-fvisibility=hidden", "-I", INCLUDE, "-I", CSRC]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build softglrender_gb300")


def _sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _deps_mtime() -> float:
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(INCLUDE, "softgl_cuda.h"), __file__]
    return max(os.path.getmtime(f) for f in files)


def build(force: bool = False, verbose: bool = False, extra_flags=()) -> str:
    """Compile and link the library if any source is newer than it. Returns its path."""
    os.makedirs(OUT, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _deps_mtime():
        return LIB
    nvcc = _nvcc()
    srcs = _sources()

    def compile_one(src):
        obj = os.path.join(OUT, os.path.basename(src).replace(".cu", ".o"))
        cmd = [nvcc, *FLAGS, *extra_flags, "-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {os.path.basename(src)}:\n{r.stderr[-4000:]}")
        if verbose:
            sys.stderr.write(r.stderr)
        return obj

    workers = min(len(srcs), max(1, os.cpu_count() or 1))
    with cf.ThreadPoolExecutor(max_workers=workers) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = LIB + ".tmp"
    r = subprocess.run([nvcc, ARCH, "-shared", "-o", tmp, *objs], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr[-4000:]}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
