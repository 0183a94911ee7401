"""ard_read_field_noalloc against ard_read_field and the FP64 oracle.

The no-allocation readout serves callers that cannot allocate device memory
(code inside another framework's memory pool, or whose allocator is owned by
someone else).  It must give the same field as the ordinary readout and as
the oracle's inverse transform, on two calls in a row over a stepping
simulation, on the context's stream and on a caller's stream, for small
partitions (one 64 x 64 tile per pass) and for one whose every axis spans
several ragged tiles.  Oversized partitions are refused before anything is
queued or written.  This file sorts last so that a run stopping at the first
failure has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

import ard_gb300 as A
from oracle import oracle as O

pytestmark = pytest.mark.gpu

H, C0 = 0.1, 343.0
DT = float(np.float32(0.5 * H / (C0 * np.sqrt(3.0))))


def _ptr(t):
    return C.cast(t.data_ptr(), C.POINTER(C.c_float))


def _pulse(n):
    return (1e3 * np.exp(-((np.arange(n) - 12.0) ** 2) / 18.0)).astype(np.float32)


@pytest.mark.parametrize("air,src,caller_stream", [
    ([(0, 0, 0, 20, 16, 12), (20, 4, 0, 14, 10, 12)], (6, 7, 6), False),
    ([(0, 0, 0, 130, 70, 66)], (40, 30, 20), True),
])
def test_read_field_noalloc_matches_read_field(air, src, caller_stream):
    torch = pytest.importorskip("torch")
    scene = A.build_scene(air, [src], [], H, DT, C0, 5)
    sim = A.Simulation(scene, max_steps=64)
    sim.set_source_series(0, _pulse(64))
    flat = O.make_flat_scene(air, [src], [], dict(dh=H, dt=DT, c0=C0, pml_layers=5))
    ref = O.OracleSim(flat, "f64")
    ref.set_source_series(0, _pulse(64))
    stream = torch.cuda.Stream() if caller_stream else None
    for steps in (20, 15):  # two calls in a row, the state moving on in between
        sim.run(steps)
        ref.step(steps)
        for part in range(len(air)):
            want = sim.field(part)
            oracle = ref.field(part)[0]
            q = scene.partitions[part]
            buf = torch.full((q[7] * q[6] * q[5],), float("nan"), dtype=torch.float32, device="cuda")
            rc = A.lib().ard_read_field_noalloc(sim._h, 0, part, _ptr(buf),
                                                C.c_void_p(stream.cuda_stream) if stream else None)
            assert rc == A.ARD_OK, A._err(sim._h)
            if stream:
                stream.synchronize()
            sim.synchronize()
            got = buf.cpu().numpy().reshape(q[7], q[6], q[5])
            assert np.all(np.isfinite(got))
            scale = np.abs(oracle).max()
            assert scale > 0
            assert np.abs(got - want).max() <= 1e-6 * np.abs(want).max()
            assert np.abs(got - oracle).max() <= 1e-4 * scale
    sim.close()


@pytest.mark.parametrize("box", [(0, 0, 0, 200, 200, 120),   # 4.8 M cells: over the cell limit
                                 (0, 0, 0, 8, 8, 1025)])      # an extent over 1024
def test_read_field_noalloc_refuses_oversized(box):
    torch = pytest.importorskip("torch")
    big = A.build_scene([box], [(4, 4, 6)], [], H, DT, C0, 5)
    sim = A.Simulation(big, max_steps=4)
    dummy = torch.zeros(16, dtype=torch.float32, device="cuda")
    rc = A.lib().ard_read_field_noalloc(sim._h, 0, 0, _ptr(dummy), None)
    assert rc == 6  # ARD_ERR_RANGE
    sim.synchronize()
    assert torch.count_nonzero(dummy).item() == 0   # nothing written
    sim.close()
