"""Build the engine's shared library librc.so in-tree for sm_103a.

Host translation units are compiled with g++, CUDA units with nvcc for
sm_103a only, in parallel, then linked into radiancecascade_gb300/librc.so
(git-ignored).  Rebuilds only when a source is newer than the library.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OBJ = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "librc.so")
# the checked build (-DRC_CHECKED): bounds-tested kernels, see csrc/rc_check.cuh
OBJ_CHECKED = os.path.join(PKG, "_build_checked")
LIB_CHECKED = os.path.join(PKG, "librc_checked.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else (shutil.which("nvcc") or "nvcc")


def _sources():
    cu = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    cpp = sorted(glob.glob(os.path.join(CSRC, "*.cpp")))
    hdr = sorted(glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh"))
                 + [os.path.join(ROOT, "include", "rc.h")])
    return cu, cpp, hdr


def _compile(src: str, checked: bool = False) -> str:
    obj = OBJ_CHECKED if checked else OBJ
    defs = ["-DRC_CHECKED"] if checked else []
    out = os.path.join(obj, os.path.basename(src) + ".o")
    if src.endswith(".cu"):
        cmd = [_nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", *defs, "-Xcompiler", "-fPIC,-ffp-contract=off",
               "-Xptxas", "-v", "-c", src, "-o", out]
    else:
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", *defs,
               "-I", os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include"),
               "-c", src, "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    log = os.path.join(obj, os.path.basename(src) + ".log")
    with open(log, "w") as f:
        f.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
    if r.returncode != 0:
        raise RuntimeError("compile failed: %s\n%s" % (" ".join(cmd), r.stderr[-4000:]))
    return out


def build(force: bool = False, verbose: bool = False, checked: bool = False) -> str:
    """Builds librc.so, or with `checked` librc_checked.so (same sources with
    RC_CHECKED: every instrumented buffer access is tested before it is made)."""
    lib, obj = (LIB_CHECKED, OBJ_CHECKED) if checked else (LIB, OBJ)
    cu, cpp, hdr = _sources()
    srcs = cu + cpp
    if not force and os.path.exists(lib):
        t = os.path.getmtime(lib)
        if all(os.path.getmtime(s) <= t for s in srcs + hdr + [__file__]):
            return lib
    os.makedirs(obj, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=max(2, min(len(srcs), os.cpu_count() or 2))) as ex:
        objs = list(ex.map(lambda src: _compile(src, checked), srcs))
    tmp = lib + ".tmp%d" % os.getpid()
    cmd = [_nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed: %s\n%s" % (" ".join(cmd), r.stderr[-4000:]))
    os.replace(tmp, lib)
    if verbose:
        for s in srcs:
            with open(os.path.join(obj, os.path.basename(s) + ".log")) as f:
                sys.stdout.write(f.read())
    return lib


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv, checked="--checked" in sys.argv))
