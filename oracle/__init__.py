"""Test infrastructure: the checkers the CUDA renderer is compared against. Nothing in the
product (softglrender_gb300) imports this package; only tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline arm do.

Two checkers export the same C ABI as the product (include/softgl_cuda.h):

* `reference()`: the unmodified reference RendererSoft compiled from the reference sources by
  oracle/ref/Makefile into oracle/_ref/ (symbol prefix `sglr_`). Buildable only where the
  reference tree is present on an x86-64 host; parity of everything else is pinned to it.
* `restatement()`: oracle/softgl_oracle.cpp, a portable C++ restatement of the same pipeline
  (prefix `sglo_`), compiled by `build()` on any host, including the Arm GPU machine.
"""
from __future__ import annotations

import ctypes
import os
import platform
import subprocess
from typing import Optional

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
ORACLE_SO = os.path.join(HERE, "_build", "libsoftgl_oracle.so")


def build(verbose: bool = False) -> str:
    """Compile the C++ restatement (and, where the reference tree exists on x86-64, the
    reference-backed checkers). Returns the restatement's path."""
    os.makedirs(os.path.dirname(ORACLE_SO), exist_ok=True)
    src = os.path.join(HERE, "softgl_oracle.cpp")
    inc = os.path.join(os.path.dirname(HERE), "include")
    if (not os.path.exists(ORACLE_SO)) or os.path.getmtime(ORACLE_SO) < os.path.getmtime(src):
        cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math",
               "-pthread", "-I", inc, src, "-o", ORACLE_SO]
        if platform.machine() in ("x86_64", "AMD64"):
            cmd.insert(1, "-mfma")   # hardware fmaf (same results as the libm routine, faster)
        subprocess.run(cmd, check=True, capture_output=not verbose)
    if platform.machine() in ("x86_64", "AMD64") and _have_reference_tree():
        subprocess.run(["make", "-s", "-C", os.path.join(HERE, "ref"), f"OUT={REF_DIR}", "-j4"],
                       check=True, capture_output=not verbose)
    return ORACLE_SO


def _have_reference_tree() -> bool:
    """Whether the reference sources are present (oracle/ref/Makefile decides where they lie;
    SOFTGL_REFERENCE_TREE overrides it)."""
    r = subprocess.run(["make", "-s", "-C", os.path.join(HERE, "ref"), "have-ref"], capture_output=True)
    return r.returncode == 0


def reference_tree() -> Optional[str]:
    """The reference tree's root when its sources are present, else None."""
    if not _have_reference_tree():
        return None
    r = subprocess.run(["make", "-s", "-C", os.path.join(HERE, "ref"), "print-ref"], capture_output=True, text=True)
    return r.stdout.strip() or None


def _lib(path: str, prefix: str):
    from softglrender_gb300.api import Library
    return Library(ctypes.CDLL(path), prefix)


def restatement():
    if not os.path.exists(ORACLE_SO):
        build()
    return _lib(ORACLE_SO, "sglo_")


def reference(variant: str = "") -> Optional[object]:
    """The reference-backed checker, or None where it cannot be built (no reference tree/x86)."""
    name = "libsoftgl_ref" + (("_" + variant) if variant else "") + ".so"
    path = os.path.join(REF_DIR, name)
    if not os.path.exists(path):
        return None
    return _lib(path, "sglr_")
