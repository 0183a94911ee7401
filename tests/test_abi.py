"""The C-ABI library loads on the host and exports every declared symbol."""
import os
import re

import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "ard_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(ard_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_boundary():
    names = declared_functions()
    for must in ("ard_create", "ard_step", "ard_read_recorders", "ard_read_field", "ard_adjoint",
                 "ard_set_source_series", "ard_set_initial_pressure", "ard_set_pml_scale",
                 "ard_last_error", "ard_destroy", "ard_scene_build", "ard_scene_import"):
        assert must in names


def test_library_exports_every_declared_symbol():
    import ard_gb300
    lib = ard_gb300.lib()
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    assert lib.ard_abi_version() == 1
    # the Python signatures table covers the whole header
    assert set(declared_functions()) == set(ard_gb300.SIGNATURES)


def test_create_without_gpu_fails_loudly():
    """On a host without an sm_103a device, stepping refuses: no CPU fallback."""
    import ard_gb300 as A
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        pytest.skip("a GPU is present")
    sc = A.build_scene([(0, 0, 0, 12, 12, 12)], [(6, 6, 6)], [], 0.1, 1e-4, 343.0, 5)
    with pytest.raises(A.ArdError) as e:
        A.Simulation(sc)
    assert e.value.code == 7  # ARD_ERR_NOGPU
