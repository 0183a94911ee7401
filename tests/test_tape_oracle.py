"""The FP64 autograd tape (oracle/tape_oracle.py) against the C oracle's FP64
forward: same recorder signals to rounding, with an initial pressure and
non-unit PML face scales.  CPU only."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import oracle as O
from oracle.tape_oracle import TapeOracle

DH, C0 = 0.1, 343.0
DT = float(np.float32(0.5 * DH / (C0 * np.sqrt(3.0))))
AIR = [(0, 0, 0, 16, 14, 12), (16, 1, 0, 12, 12, 12)]
SOURCES = [(4, 5, 5), (20, 6, 4)]
RECORDERS = [(8, 6, 6), (10, 8, 7), (22, 7, 6)]


def scene():
    return O.make_flat_scene(AIR, SOURCES, RECORDERS, dict(dh=DH, dt=DT, c0=C0, pml_layers=5))


def test_tape_forward_matches_c_oracle():
    flat = scene()
    T = 30
    rng = np.random.default_rng(0)
    series = rng.standard_normal((len(SOURCES), T)).astype(np.float32)
    p0 = rng.standard_normal((12, 14, 16))
    scale = np.array([1.0, 0.75, 1.25, 1.0, 0.5, 1.5])
    ref = O.OracleSim(flat, "f64")
    for i in range(len(SOURCES)):
        ref.set_source_series(i, series[i])
    ref.set_pml_scale(scale)
    ref.set_initial_pressure(0, p0)
    ref.step(T)
    want = ref.recorders()
    tape = TapeOracle(flat)
    got = tape.run(torch.tensor(series, dtype=torch.float64), T, p0={0: torch.tensor(p0)},
                   scale6=torch.tensor(scale)).numpy()
    for r in range(want.shape[1]):
        assert np.linalg.norm(got[:, r] - want[:, r]) <= 1e-11 * np.linalg.norm(want[:, r]), r
