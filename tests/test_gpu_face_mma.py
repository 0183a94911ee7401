"""Tensor-core face transforms (split-TF32 tcgen05 passes) against the oracle.

FP32 contexts whose face layers take the two-pass form run the four passes
of the 2D face transforms on the tensor cores.  ARD_FACE_TWO_PASS=1 forces
that form on small scenes, so the FP64 C oracle and the reference's own
recorder signals check it quickly.  The split product keeps FP32-level
accuracy: the tensor-core path must agree with the fused CUDA-core path to
well inside the FP32 bar (1e-5 relative L2 where the bar is 1e-4).

The largest c4 partition (232 x 178 x 300 cells, faces of 300 rows) checks
the two-pass face transforms at c4 size: FP64 GPU (CUDA-core passes in
double) against the FP64 C oracle to 1e-10 at a recorder and to the float
rounding of the field readout, and the FP32 tensor-core run against that
FP64 run.
"""
import numpy as np
import pytest

import ard_gb300 as A
from helpers import load_run, rel_l2
from oracle import oracle as O

pytestmark = pytest.mark.gpu

F32_TOL = 1e-4


def _run(air, srcs, recs, series, T, dh, dt, c0, pml, precision=A.PREC_F32):
    sim = A.Simulation(A.build_scene(air, srcs, recs, dh, dt, c0, pml), precision=precision, max_steps=T)
    for i, s in enumerate(series):
        sim.set_source_series(i, s[:T])
    sim.run(T)
    return sim


@pytest.mark.parametrize("name", ["multi4", "scene2_gauss", "quirk_run"])
def test_tensor_core_faces_match_reference(name, monkeypatch):
    """Reference-build goldens (multi-partition scenes with interfaces and
    PML): the forced two-pass tensor-core faces within the FP32 bar of the
    reference CPU solver and within 1e-5 of the fused CUDA-core faces."""
    g = load_run(name)
    sc = g["scene"]
    p = sc["params"]
    fused = _run(sc["air"], sc["sources"], sc["recorders"], g["sources"], sc["steps"], p["dh"], p["dt"], p["c0"],
                 p["pml_layers"])
    assert "faces fused" in fused.layout
    monkeypatch.setenv("ARD_FACE_TWO_PASS", "1")
    mma = _run(sc["air"], sc["sources"], sc["recorders"], g["sources"], sc["steps"], p["dh"], p["dt"], p["c0"],
               p["pml_layers"])
    assert "faces tensor-core" in mma.layout
    got, base, want = mma.recorders(f64=True), fused.recorders(f64=True), g["recorders"]
    for r in range(want.shape[1]):
        if np.isnan(want[0, r]) or np.abs(want[:, r]).max() == 0:
            continue
        assert rel_l2(got[:, r], want[:, r]) < F32_TOL, (name, r)
        assert rel_l2(got[:, r], base[:, r]) < 1e-5, (name, r)
    # fields against the scene's largest value: a quiet partition's FP32
    # rounding is set by the loudest field that reaches it through the interfaces
    fields = [(mma.field(part), fused.field(part)) for part in range(len(sc["air"]))]
    scale = max(max(np.abs(b).max() for _, b in fields), 1e-30)
    for part, (a, b) in enumerate(fields):
        assert np.abs(a - b).max() <= 1e-5 * scale, part


def test_tensor_core_faces_ragged_two_partitions(monkeypatch):
    """Extents that are not multiples of 4 (scalar staging of the data rows,
    partial M, N and K tiles) in two partitions joined by an interface; FP32
    tensor-core passes against the FP64 C oracle."""
    monkeypatch.setenv("ARD_FACE_TWO_PASS", "1")
    dh, c0 = 0.1, 343.0
    dt = float(np.float32(0.5 * dh / (c0 * np.sqrt(3.0))))
    air = [(0, 0, 0, 141, 133, 13), (141, 5, 0, 21, 131, 13)]
    srcs, recs = [(136, 60, 6)], [(130, 58, 6), (147, 62, 7)]
    T = 60
    series = [(np.hanning(T) * 1e3).astype(np.float32)]
    flat = O.make_flat_scene(air, srcs, recs, dict(dh=dh, dt=dt, c0=c0, pml_layers=5))
    ref = O.OracleSim(flat, "f64")
    ref.set_source_series(0, series[0])
    ref.step(T)
    want = ref.recorders()
    sim = _run(air, srcs, recs, series, T, dh, dt, c0, 5)
    assert "faces tensor-core" in sim.layout
    got = sim.recorders(f64=True)
    for r in range(want.shape[1]):
        if np.abs(want[:, r]).max() > 0:
            assert rel_l2(got[:, r], want[:, r]) < 1e-5, r
    for part in range(2):
        w = ref.field(part)[0]
        assert np.abs(sim.field(part) - w).max() <= 1e-5 * np.abs(w).max(), part


def test_c4_partition_faces():
    """The largest c4 partition (232 x 178 x 300, h = 0.04 m, 10-cell PML),
    12 steps, a recorder 2 cells from the source: FP64 two-pass faces against
    the FP64 C oracle, recorder to 1e-10 relative L2 and field to the float
    rounding of ard_read_field's output (1e-7 of the field's maximum); FP32
    tensor-core faces against the FP64 GPU run within 5e-6 of the field's
    maximum and within the FP32 bar at the recorder."""
    dh, c0 = float(np.float32(0.04)), 343.0
    dt = float(np.float32(0.5 * 0.04 / (c0 * np.sqrt(3.0))))
    air, srcs, recs = [(0, 0, 0, 232, 178, 300)], [(116, 89, 150)], [(118, 90, 150)]
    T = 12
    series = [(np.hanning(T) * 1e3).astype(np.float32)]
    flat = O.make_flat_scene(air, srcs, recs, dict(dh=dh, dt=dt, c0=c0, pml_layers=10))
    ref = O.OracleSim(flat, "f64")
    ref.set_source_series(0, series[0])
    ref.step(T)
    want_rec = ref.recorders()[:, 0]
    want = ref.field(0)[0]
    ref.close()
    f64 = _run(air, srcs, recs, series, T, dh, dt, c0, 10, precision=A.PREC_F64)
    assert "faces gemm" in f64.layout
    got64 = f64.field(0).astype(np.float64)
    rec64 = f64.recorders(f64=True)[:, 0]
    f64.close()
    scale = np.abs(want).max()
    assert scale > 0
    assert np.abs(got64 - want).max() <= 1e-7 * scale
    assert rel_l2(rec64, want_rec) < 1e-10
    f32 = _run(air, srcs, recs, series, T, dh, dt, c0, 10)
    assert "faces tensor-core" in f32.layout
    err = np.abs(f32.field(0) - got64).max() / scale
    rec_err = rel_l2(f32.recorders(f64=True)[:, 0], rec64)
    print(f"c4 partition, {T} steps: FP32 tensor-core field error {err:.2e}, recorder {rec_err:.2e}")
    assert err < 5e-6
    assert rec_err < F32_TOL
