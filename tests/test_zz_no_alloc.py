"""ard_read_field_noalloc against ard_read_field.

The no-allocation readout serves callers that cannot allocate device memory
(code inside another framework's memory pool, or whose allocator is owned by
someone else).  It must give the same field as the ordinary readout, on two
calls in a row over a stepping simulation.  This file sorts last so that a
run stopping at the first failure has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

import ard_gb300 as A

pytestmark = pytest.mark.gpu


def test_read_field_noalloc_matches_read_field():
    torch = pytest.importorskip("torch")
    h, c0 = 0.1, 343.0
    dt = float(np.float32(0.5 * h / (c0 * np.sqrt(3.0))))
    scene = A.build_scene([(0, 0, 0, 20, 16, 12), (20, 4, 0, 14, 10, 12)], [(6, 7, 6)], [(10, 8, 6)],
                          h, dt, c0, 5)
    sim = A.Simulation(scene, max_steps=64)
    sim.set_source_series(0, (1e3 * np.exp(-((np.arange(64) - 12.0) ** 2) / 18.0)).astype(np.float32))
    for steps in (20, 15):  # two calls in a row, the state moving on in between
        sim.run(steps)
        for part in (0, 1):
            want = sim.field(part)
            q = scene.partitions[part]
            buf = torch.full((q[7] * q[6] * q[5],), float("nan"), dtype=torch.float32, device="cuda")
            rc = A.lib().ard_read_field_noalloc(sim._h, 0, part, C.cast(buf.data_ptr(), C.POINTER(C.c_float)), None)
            assert rc == A.ARD_OK, A._err(sim._h)
            sim.synchronize()
            got = buf.cpu().numpy().reshape(q[7], q[6], q[5])
            assert np.all(np.isfinite(got))
            assert np.abs(got - want).max() <= 1e-6 * np.abs(want).max()
    # beyond the fixed scratch: refused with a range error, nothing written
    big = A.build_scene([(0, 0, 0, 200, 200, 120)], [(6, 7, 6)], [], h, dt, c0, 5)
    sim_big = A.Simulation(big, max_steps=4)
    dummy = torch.zeros(4, dtype=torch.float32, device="cuda")
    rc = A.lib().ard_read_field_noalloc(sim_big._h, 0, 0, C.cast(dummy.data_ptr(), C.POINTER(C.c_float)), None)
    assert rc == 6  # ARD_ERR_RANGE
