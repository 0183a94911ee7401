"""Build recipe of libard_gb300.so (sm_103a kernels + host scene builder).

Each translation unit compiles in parallel; the shared library is written
next to this file so the package loads it in-tree.
"""
from __future__ import annotations

import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)                      # ard-simulator_gb300/
REPO = os.path.dirname(ROOT)
CSRC = os.path.join(ROOT, "csrc")
INCLUDE = os.path.join(REPO, "include")
BUILD = os.path.join(ROOT, "_build")
LIB = os.path.join(PKG, "libard_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_SOURCES = ["ard_engine.cu", "ard_layout.cu", "ard_adjoint.cu", "ard_noalloc.cu", "ard_output.cu", "ard_post.cu"]
CPP_SOURCES = ["ard_scene.cpp"]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _deps():
    out = [os.path.join(INCLUDE, "ard_gb300.h")]
    for f in os.listdir(CSRC):
        out.append(os.path.join(CSRC, f))
    return out


def stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(d) > t for d in _deps())


def build(force=False, verbose=False):
    """Compile every translation unit (in parallel) and link the library."""
    if not force and not stale():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    nv = nvcc()
    common = ["-std=c++17", "-O3", "-I", INCLUDE, "-I", CSRC]
    cmds, objs = [], []
    for src in CU_SOURCES:
        path = os.path.join(CSRC, src)
        if not os.path.exists(path):
            continue
        obj = os.path.join(BUILD, src + ".o")
        cmds.append([nv] + ARCH + common + ["-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off",
                                           "-Xptxas", "-v" if verbose else "-O3", "-c", path, "-o", obj])
        objs.append(obj)
    for src in CPP_SOURCES:
        path = os.path.join(CSRC, src)
        obj = os.path.join(BUILD, src + ".o")
        cmds.append(["g++", "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-I", INCLUDE, "-c", path, "-o", obj])
        objs.append(obj)
    procs = [(c, subprocess.Popen(c, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)) for c in cmds]
    failed = []
    for c, p in procs:
        out, _ = p.communicate()
        if verbose and out:
            print(out)
        if p.returncode != 0:
            failed.append((c, out))
    if failed:
        msg = "\n".join(" ".join(c) + "\n" + o for c, o in failed)
        raise RuntimeError("libard_gb300 compile failed:\n" + msg)
    tmp = LIB + ".tmp"
    subprocess.check_call([nv] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart_static", "-lrt", "-ldl", "-lpthread"])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
