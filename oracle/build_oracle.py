"""ORACLE / TEST INFRASTRUCTURE ONLY.

Build recipe for the checker libraries: liboracle.so (the C restatement in
both precisions plus the DCT) into oracle/_build/, and, when the reference
sources are present, the headless reference build into oracle/_ref/.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")
# The reference sources: ARD_REFERENCE_DIR, else where this container mounts them.
REFDIR = os.environ.get("ARD_REFERENCE_DIR", "/root/reference/ARD-simulator-190113")
REF_BIN = os.path.join(HERE, "_ref", "ard_ref")

_SOURCES = ["ard_oracle.c", "dct_fft.c"]


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def oracle_commands():
    """Shell commands (argv lists) that build liboracle.so; independent ones
    first so a caller may run them in parallel."""
    os.makedirs(BUILD, exist_ok=True)
    common = ["gcc", "-O3", "-fPIC", "-fopenmp", "-ffp-contract=off", "-std=c11", "-D_GNU_SOURCE"]
    objs = {
        "f32": (os.path.join(BUILD, "oracle_f32.o"),
                common + ["-DREAL=float", "-DSFX=_f32", "-c", os.path.join(HERE, "ard_oracle.c")]),
        "f64": (os.path.join(BUILD, "oracle_f64.o"),
                common + ["-DREAL=double", "-DSFX=_f64", "-DORACLE_DOUBLE", "-c",
                          os.path.join(HERE, "ard_oracle.c")]),
        "dct": (os.path.join(BUILD, "dct_fft.o"), common + ["-c", os.path.join(HERE, "dct_fft.c")]),
    }
    compile_cmds = [argv + ["-o", out] for out, argv in objs.values()]
    link = ["gcc", "-shared", "-fopenmp", "-o", LIB] + [o for o, _ in objs.values()] + ["-lm", "-lpthread"]
    return compile_cmds, link


def build_oracle(force=False):
    deps = [os.path.join(HERE, s) for s in _SOURCES] + [
        os.path.join(HERE, "dct_fft.h"), os.path.join(HERE, "..", "include", "ard_gb300.h")]
    if not force and not _stale(LIB, deps):
        return LIB
    compile_cmds, link = oracle_commands()
    procs = [subprocess.Popen(c) for c in compile_cmds]
    if any(p.wait() != 0 for p in procs):
        raise RuntimeError("oracle compile failed")
    subprocess.check_call(link)
    return LIB


def build_reference(force=False):
    """Headless reference build; returns the binary path or None when the
    reference sources are not on this machine."""
    if not os.path.isdir(REFDIR):
        return None
    if force or not os.path.exists(REF_BIN):
        subprocess.check_call(["make", "-s", "-j8", "-C", os.path.join(HERE, "ref_build"),
                               f"REFDIR={REFDIR}"])
    return REF_BIN


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    print(build_reference(force="--force" in sys.argv))
