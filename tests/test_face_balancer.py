"""The fused face transforms' job balancer (ard::balance_face_jobs in
ard_layout.cu) on the host: tests/face_balance_check.cpp is compiled with
g++ against the built library's own function and run; it checks the cluster
pairing, that every output slab is produced once, the one-wave stop and the
whole-list rule for long lists.  No GPU is needed."""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT

CSRC = os.path.join(ROOT, "ard-simulator_gb300", "csrc")


def test_face_balancer(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not found")
    import ard_gb300
    lib = ard_gb300.lib()
    libpath = lib._name
    libdir = os.path.dirname(os.path.abspath(libpath))
    exe = str(tmp_path / "face_balance_check")
    subprocess.check_call([gxx, "-std=c++17", "-O1", "-I", CSRC, os.path.join(ROOT, "tests", "face_balance_check.cpp"),
                           "-o", exe, "-L", libdir, "-l:" + os.path.basename(libpath), "-Wl,-rpath," + libdir])
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "face balancer ok" in r.stdout
