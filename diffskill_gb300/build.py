"""Build the sm_103a CUDA library ``libmpm_gb300.so`` in-tree with nvcc.

The translation units compile in parallel (one ``-gencode``) and link into a
shared library next to this file, which ``diffskill_gb300._lib`` loads with
ctypes.  No CMake, no torch extension machinery: the library is plain C ABI.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
REPO = os.path.dirname(HERE)
LIB = os.path.join(HERE, "libmpm_gb300.so")
BUILD_DIR = os.path.join(HERE, "_build")
SOURCES = ["mpm_capi.cu", "mpm_fwd.cu", "mpm_bwd.cu", "mpm_loss.cu", "mpm_kinematics.cu", "mpm_render.cu",
           "mpm_static.cu", "mpm_sort.cu"]
# per-file flags: the renderer rounds every FP32 operation on its own (no FMA
# contraction), as its reference arithmetic does.  The substep kernels flush
# FP32 subnormals to zero and take FP32 divides and square roots by the fast
# approximations (the SVD, the return map and the tool SDFs and contact are
# full of them; 4 % and another 3.7 % per iteration).  FP64 is unaffected.
_FAST32 = ("-ftz=true", "-prec-div=false", "-prec-sqrt=false")
EXTRA = {"mpm_render.cu": ("-fmad=false",), "mpm_fwd.cu": _FAST32, "mpm_bwd.cu": _FAST32, "mpm_static.cu": _FAST32}
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found; the CUDA toolkit is required to build diffskill_gb300")
    return exe


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files.append(os.path.join(REPO, "include", "mpm_gb300.h"))
    files.append(os.path.abspath(__file__))  # the flags
    return files


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(f) <= t for f in _deps())


def compile_one(src: str, extra=(), verbose: bool = False) -> str:
    os.makedirs(BUILD_DIR, exist_ok=True)
    obj = os.path.join(BUILD_DIR, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-c",
           os.path.join(CSRC, src), "-o", obj, *extra]
    if verbose:
        cmd += ["-Xptxas", "-v"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
    if verbose:
        sys.stderr.write(r.stderr)
    return obj


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile every CUDA source for sm_103a and link ``libmpm_gb300.so``."""
    if not force and up_to_date():
        return LIB
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: compile_one(s, EXTRA.get(s, ()), verbose=verbose), SOURCES))
    tmp = LIB + ".tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(LIB)
