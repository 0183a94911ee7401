"""GPU parity: the sm_103a path through the C ABI against the reference
(golden fixtures made by the reference build) and the oracle.

Tolerances: FP32 recorder signals within 1e-4 relative L2 of the reference
(the FP32 accuracy bar); the FP64 GPU oracle within 1e-10 of the FP64 C oracle
(same algorithm, different summation order)."""
import numpy as np
import pytest

import ard_gb300 as A
from helpers import load_run, rel_l2
from oracle import oracle as O

pytestmark = pytest.mark.gpu

F32_TOL = 1e-4
F64_TOL = 1e-10


def gpu_run(sc, series, precision=A.PREC_F32, graphs=True, steps=None, arithmetic=A.ARITH_ACCURATE):
    p = sc["params"]
    scene = A.build_scene(sc["air"], sc["sources"], sc["recorders"], p["dh"], p["dt"], p["c0"], p["pml_layers"])
    T = steps or sc["steps"]
    sim = A.Simulation(scene, precision=precision, max_steps=T, use_graphs=graphs, arithmetic=arithmetic)
    for i, s in enumerate(series):
        sim.set_source_series(i, s[:T])
    sim.run(T)
    return scene, sim


@pytest.mark.parametrize("arith", [0, 1])
@pytest.mark.parametrize("name", ["multi4", "scene2_gauss", "quirk_run"])
def test_recorders_match_reference(name, arith):
    g = load_run(name)
    sc = g["scene"]
    _, sim = gpu_run(sc, g["sources"], arithmetic=arith)
    got = sim.recorders(f64=True)
    want = g["recorders"]
    for r in range(want.shape[1]):
        if np.isnan(want[0, r]):
            continue  # recorder outside every partition in the reference run
        assert rel_l2(got[:, r], want[:, r]) < F32_TOL, (name, r)


@pytest.mark.parametrize("name", ["multi4", "quirk_run"])
def test_fields_match_oracle(name):
    g = load_run(name)
    sc = g["scene"]
    flat = O.make_flat_scene(sc["air"], sc["sources"], sc["recorders"], sc["params"])
    ref = O.OracleSim(flat, "f32")
    for i, s in enumerate(g["sources"]):
        ref.set_source_series(i, s)
    ref.step(sc["steps"])
    _, sim = gpu_run(sc, g["sources"])
    wants = [ref.field(i)[0] for i in range(len(flat["partitions"]))]
    scale = max(np.abs(w).max() for w in wants)   # near-silent PML slabs are measured against the scene's scale
    for i, want in enumerate(wants):
        got = sim.field(i)
        assert np.abs(got - want).max() / scale < 1e-4, i


@pytest.mark.parametrize("name", ["multi4", "quirk_run"])
def test_fp64_gpu_oracle_matches_fp64_c_oracle(name):
    g = load_run(name)
    sc = g["scene"]
    flat = O.make_flat_scene(sc["air"], sc["sources"], sc["recorders"], sc["params"])
    ref = O.OracleSim(flat, "f64")
    for i, s in enumerate(g["sources"]):
        ref.set_source_series(i, s)
    ref.step(sc["steps"])
    want = ref.recorders()
    _, sim = gpu_run(sc, g["sources"], precision=A.PREC_F64)
    got = sim.recorders(f64=True)
    for r in range(want.shape[1]):
        if np.abs(want[:, r]).max() > 0:
            assert rel_l2(got[:, r], want[:, r]) < F64_TOL


def test_graphs_equal_direct_launches():
    g = load_run("multi4")
    _, a = gpu_run(g["scene"], g["sources"], graphs=True)
    _, b = gpu_run(g["scene"], g["sources"], graphs=False)
    assert np.array_equal(a.recorders(f64=True), b.recorders(f64=True))


def test_reset_reproduces_bitwise_and_update_counts():
    g = load_run("multi4")
    sc = g["scene"]
    _, sim = gpu_run(sc, g["sources"])
    first = sim.recorders(f64=True)
    sim.reset()
    assert sim.time_step == 0
    assert sim.Update() == 0          # returns the pre-increment index, as Simulation::Update
    sim.run(sc["steps"] - 1)
    assert np.array_equal(sim.recorders(f64=True), first)


def test_linearity_and_time_shift():
    """The step is linear in the source series and time-invariant."""
    g = load_run("multi4")
    sc = g["scene"]
    T = sc["steps"]
    base = [np.asarray(s, np.float32) for s in g["sources"]]
    _, s1 = gpu_run(sc, base)
    r1 = s1.recorders(f64=True)
    _, s2 = gpu_run(sc, [2.0 * s for s in base])
    assert rel_l2(s2.recorders(f64=True), 2.0 * r1) < 1e-6
    k = 7
    shifted = [np.r_[np.zeros(k, np.float32), s[:T - k]] for s in base]
    _, s3 = gpu_run(sc, shifted)
    assert rel_l2(s3.recorders(f64=True)[k:], r1[:T - k]) < 1e-5


def test_batched_scenes_equal_individual_runs():
    """One context holding three scenes gives each scene's own answer: in
    FP64 to round-off (tiling differs, the mathematics does not), and the
    FP32 batch stays within 1e-4 of it."""
    from ard_gb300 import configs as K
    cfg = K.config("c2", steps=120)
    picks = cfg["scenes"][:3]
    h = float(np.float32(cfg["h"]))
    scenes = [A.build_scene(s["air"], s["sources"], s["recorders"], h, cfg["dt"], cfg["c0"], cfg["pml"]) for s in picks]

    def batch_run(prec):
        sim = A.Simulation(scenes, max_steps=120, precision=prec)
        for i, s in enumerate(picks):
            sim.set_source_series(0, s["series"][0], scene=i)
        sim.run(120)
        return sim

    b64, b32 = batch_run(A.PREC_F64), batch_run(A.PREC_F32)
    for i, s in enumerate(picks):
        one = A.Simulation(scenes[i], max_steps=120, precision=A.PREC_F64)
        one.set_source_series(0, s["series"][0])
        one.run(120)
        ref = one.recorders(f64=True)
        assert rel_l2(b64.recorders(scene=i, f64=True), ref) < 1e-10
        assert rel_l2(b32.recorders(scene=i, f64=True), ref) < 1e-4
    allrec = b32.recorders(scene=-1, f64=True)
    assert allrec.shape == (120, sum(len(s["recorders"]) for s in picks))


def test_initial_pressure_round_trip():
    sc = A.build_scene([(0, 0, 0, 14, 11, 9)], [(5, 5, 5)], [], 0.1, 1e-4, 343.0, 5)
    rng = np.random.default_rng(0)
    p0 = rng.standard_normal((9, 11, 14)).astype(np.float32)
    for prec in (A.PREC_F32, A.PREC_F64):
        sim = A.Simulation(sc, precision=prec, max_steps=16)
        sim.set_initial_pressure(0, p0)
        got = sim.field(0)
        tol = 1e-5 if prec == A.PREC_F32 else 1e-7
        assert np.abs(got - p0).max() < tol * np.abs(p0).max()


def test_initial_pressure_dynamics_match_oracle():
    air, src, rec = [(0, 0, 0, 14, 12, 12), (14, 2, 0, 10, 8, 12)], [(5, 5, 5)], [(8, 6, 6)]
    h, c = 0.1, 343.0
    dt = float(np.float32(0.5 * h / (c * np.sqrt(3))))
    params = dict(dh=h, dt=dt, c0=c, pml_layers=5)
    flat = O.make_flat_scene(air, src, rec, params)
    rng = np.random.default_rng(1)
    p0 = rng.standard_normal((12, 12, 14))
    ref = O.OracleSim(flat, "f64")
    ref.set_initial_pressure(0, p0)
    ref.step(50)
    sim = A.Simulation(A.build_scene(air, src, rec, h, dt, c, 5), precision=A.PREC_F64, max_steps=50)
    sim.set_initial_pressure(0, p0.astype(np.float32))
    sim.run(50)
    # the float32 upload of p0 limits agreement to ~1e-7
    assert rel_l2(sim.recorders(f64=True)[:, 0], ref.recorders()[:, 0]) < 1e-6


def test_errors_are_reported():
    g = load_run("multi4")
    _, sim = gpu_run(g["scene"], g["sources"], steps=10)
    with pytest.raises(A.ArdError) as e:
        sim.recorders(t0=0, nt=11)
    assert e.value.code == 6
    with pytest.raises(A.ArdError):
        sim.set_source_series(5, np.zeros(4, np.float32))
    with pytest.raises(A.ArdError):
        sim.set_initial_pressure(0, np.zeros((20, 20, 20), np.float32))  # after stepping: state error
    with pytest.raises(A.ArdError):
        sim.field(99)


def test_contexts_with_different_layer_sizes_interleave():
    """Kernel launch attributes are process-wide: contexts of different face
    sizes must run interleaved (a small context configured last must not
    break a larger one)."""
    dh, c0 = 0.1, 343.0
    dt = 0.5 * dh / (c0 * np.sqrt(3.0))
    big = A.Simulation(A.build_scene([(0, 0, 0, 96, 64, 40)], [(10, 10, 10)], [(20, 20, 20)], dh, dt, c0, 5),
                       max_steps=64)
    small = A.Simulation(A.build_scene([(0, 0, 0, 16, 16, 16)], [(5, 5, 5)], [(8, 8, 8)], dh, dt, c0, 5),
                         max_steps=64)
    for sim in (big, small):
        sim.set_source_series(0, np.hanning(64).astype(np.float32))
    small.run(8)
    big.run(8)
    small.run(8)
    big.run(40)
    assert big.time_step == 48 and small.time_step == 16
    assert np.isfinite(big.recorders()).all() and np.abs(big.recorders()).max() > 0


def test_autotuned_context_matches_default():
    """The autotuner only changes the tiling (summation order): same recorders
    to rounding, and it reports the candidates it timed."""
    g = load_run("multi4")
    sc = g["scene"]
    p = sc["params"]
    scene = A.build_scene(sc["air"], sc["sources"], sc["recorders"], p["dh"], p["dt"], p["c0"], p["pml_layers"])
    T = sc["steps"]
    out = []
    for tune in (False, True):
        sim = A.Simulation(scene, max_steps=T, autotune=tune)
        for i, s in enumerate(g["sources"]):
            sim.set_source_series(i, s[:T])
        sim.run(T)
        out.append(sim.recorders(f64=True))
        if tune:
            assert sim.layout.startswith("autotuned") and "us/step" in sim.layout
            assert sim.time_step == T
    assert rel_l2(out[1][:, 0], out[0][:, 0]) < 1e-5


def test_gemm_face_transforms_fp64_match_oracle():
    """A face of 140 rows is beyond the fused face kernel (128 rows): the
    two-pass GEMM transforms run; FP64 GPU against the FP64 C oracle to
    1e-10."""
    dh, c0 = 0.1, 343.0
    dt = float(np.float32(0.5 * dh / (c0 * np.sqrt(3.0))))
    air, srcs, recs = [(0, 0, 0, 140, 140, 16)], [(30, 40, 8)], [(60, 55, 8), (20, 80, 7)]
    T = 30
    series = (np.hanning(T) * 1e3).astype(np.float32)
    flat = O.make_flat_scene(air, srcs, recs, dict(dh=dh, dt=dt, c0=c0, pml_layers=5))
    ref = O.OracleSim(flat, "f64")
    ref.set_source_series(0, series)
    ref.step(T)
    want = ref.recorders()
    sim = A.Simulation(A.build_scene(air, srcs, recs, dh, dt, c0, 5), precision=A.PREC_F64, max_steps=T)
    assert "gemm" in sim.layout
    sim.set_source_series(0, series)
    sim.run(T)
    got = sim.recorders(f64=True)
    for r in range(want.shape[1]):
        assert rel_l2(got[:, r], want[:, r]) < F64_TOL, r


def test_fused_face_kernel_fp64_large_and_ragged_faces():
    """The fused face kernel in FP64 near its shared-memory limit: 80-row
    faces (two rows per thread, split 16-column jobs) and ragged extents (rows
    not a multiple of 4: scalar staging); against the FP64 C oracle to 1e-10."""
    dh, c0 = 0.1, 343.0
    dt = float(np.float32(0.5 * dh / (c0 * np.sqrt(3.0))))
    for air, srcs, recs in (([(0, 0, 0, 80, 80, 16)], [(30, 40, 8)], [(60, 55, 8), (20, 70, 7)]),
                            ([(0, 0, 0, 97, 61, 13)], [(40, 30, 6)], [(50, 33, 6), (20, 40, 7)])):
        T = 30
        series = (np.hanning(T) * 1e3).astype(np.float32)
        flat = O.make_flat_scene(air, srcs, recs, dict(dh=dh, dt=dt, c0=c0, pml_layers=5))
        ref = O.OracleSim(flat, "f64")
        ref.set_source_series(0, series)
        ref.step(T)
        want = ref.recorders()
        sim = A.Simulation(A.build_scene(air, srcs, recs, dh, dt, c0, 5), precision=A.PREC_F64, max_steps=T)
        assert "fused" in sim.layout
        sim.set_source_series(0, series)
        sim.run(T)
        got = sim.recorders(f64=True)
        for r in range(want.shape[1]):
            assert rel_l2(got[:, r], want[:, r]) < F64_TOL, (air, r)


def test_gemm_face_transforms_ragged_fp64_match_oracle():
    """GEMM face passes on extents that are not multiples of 4 (scalar
    cp.async staging of both operand layouts, partial tiles) in a two-partition
    scene with an interface; FP64 GPU against the FP64 C oracle to 1e-10."""
    dh, c0 = 0.1, 343.0
    dt = float(np.float32(0.5 * dh / (c0 * np.sqrt(3.0))))
    air = [(0, 0, 0, 141, 133, 13), (141, 5, 0, 21, 131, 13)]
    srcs, recs = [(136, 60, 6)], [(130, 58, 6), (147, 62, 7)]   # both reached through the interface region
    T = 60
    series = (np.hanning(T) * 1e3).astype(np.float32)
    flat = O.make_flat_scene(air, srcs, recs, dict(dh=dh, dt=dt, c0=c0, pml_layers=5))
    ref = O.OracleSim(flat, "f64")
    ref.set_source_series(0, series)
    ref.step(T)
    want = ref.recorders()
    sim = A.Simulation(A.build_scene(air, srcs, recs, dh, dt, c0, 5), precision=A.PREC_F64, max_steps=T)
    assert "gemm" in sim.layout
    sim.set_source_series(0, series)
    sim.run(T)
    got = sim.recorders(f64=True)
    for r in range(want.shape[1]):
        if np.abs(want[:, r]).max() > 0:
            assert rel_l2(got[:, r], want[:, r]) < F64_TOL, r


def test_write_outputs_in_reference_format(tmp_path):
    """response_<r>.txt / source_<s>.txt: one value per line, the recorder
    history and the injected series (output/README.md)."""
    g = load_run("scene2_gauss")
    sc = g["scene"]
    scene, sim = gpu_run(sc, g["sources"])
    T = sim.time_step
    sim.write_outputs(str(tmp_path))
    rec = sim.recorders()
    for r in range(rec.shape[1]):
        vals = np.loadtxt(tmp_path / f"response_{r}.txt")
        assert vals.shape == (T,)
        np.testing.assert_allclose(vals, rec[:, r], rtol=1e-5, atol=1e-30)
    src = np.loadtxt(tmp_path / "source_0.txt")
    np.testing.assert_allclose(src, g["sources"][0][:T], rtol=1e-5)


def test_edge_cases_empty_and_ragged():
    """Zero-step runs, a scene without sources or recorders, odd extents
    (not multiples of 4 or 8), steps past max_steps (no history, no source)."""
    dh, c0 = 0.1, 343.0
    dt = 0.5 * dh / (c0 * np.sqrt(3.0))
    # no sources, no recorders: the state stays exactly zero
    sim = A.Simulation(A.build_scene([(0, 0, 0, 13, 11, 9)], [], [], dh, dt, c0, 5), max_steps=16)
    sim.run(0)
    assert sim.time_step == 0
    sim.run(20)                                   # past max_steps: stepping continues
    assert sim.time_step == 20
    assert np.all(sim.field(0) == 0)
    # ragged extents with a source and recorders; FP32 against the FP64 C oracle
    air, srcs, recs = [(0, 0, 0, 17, 13, 15), (17, 1, 0, 11, 12, 15)], [(5, 6, 7)], [(8, 6, 7), (23, 7, 7)]
    T = 40
    series = (np.hanning(T) * 1e3).astype(np.float32)
    flat = O.make_flat_scene(air, srcs, recs, dict(dh=dh, dt=float(np.float32(dt)), c0=c0, pml_layers=5))
    ref = O.OracleSim(flat, "f64")
    ref.set_source_series(0, series)
    ref.step(T)
    want = ref.recorders()
    sim = A.Simulation(A.build_scene(air, srcs, recs, dh, float(np.float32(dt)), c0, 5), max_steps=T)
    sim.set_source_series(0, series)
    sim.run(T)
    got = sim.recorders(f64=True)
    for r in range(want.shape[1]):
        if np.abs(want[:, r]).max() > 0:
            assert rel_l2(got[:, r], want[:, r]) < F32_TOL, r


@pytest.mark.parametrize("path", ["tensor-core", "gemm"])
def test_gemm_face_transforms_fp32_match_oracle(path, monkeypatch):
    """200 x 200 faces in FP32 exceed the fused kernel's 128 rows: the
    two-pass face transforms run, on the tensor cores (default) or on the
    CUDA cores (ARD_FACE_MMA=0); FP32 against the FP64 C oracle within the
    FP32 bar (recorders a few cells from the source, reached in time)."""
    if path == "gemm":
        monkeypatch.setenv("ARD_FACE_MMA", "0")
    dh, c0 = 0.1, 343.0
    dt = float(np.float32(0.5 * dh / (c0 * np.sqrt(3.0))))
    air, srcs, recs = [(0, 0, 0, 200, 200, 16)], [(60, 80, 8)], [(66, 82, 8), (55, 77, 7)]
    T = 60
    series = (np.hanning(T) * 1e3).astype(np.float32)
    flat = O.make_flat_scene(air, srcs, recs, dict(dh=dh, dt=dt, c0=c0, pml_layers=5))
    ref = O.OracleSim(flat, "f64")
    ref.set_source_series(0, series)
    ref.step(T)
    want = ref.recorders()
    sim = A.Simulation(A.build_scene(air, srcs, recs, dh, dt, c0, 5), max_steps=T)
    assert "faces " + path in sim.layout
    sim.set_source_series(0, series)
    sim.run(T)
    got = sim.recorders(f64=True)
    for r in range(want.shape[1]):
        assert rel_l2(got[:, r], want[:, r]) < F32_TOL, r


@pytest.mark.parametrize("arith", [A.ARITH_ACCURATE, A.ARITH_REFERENCE])
def test_batched_c2_scenes_match_reference(arith):
    """Three c2 scenes (seeded guillotine decompositions, h = 0.05 m, 7-11 air
    partitions each) in ONE batched FP32 context, every scene's recorders
    within the FP32 bar of the reference's own run of that scene
    (tests/golden/make_golden.py --c2), in both arithmetic modes."""
    runs = [(n, load_run(n)) for n in ("c2scene0", "c2scene1", "c2scene3")]
    runs = [(n, g) for n, g in runs if g is not None]
    if not runs:
        pytest.skip("c2 goldens not generated")
    scenes = []
    for _, g in runs:
        sc, p = g["scene"], g["scene"]["params"]
        scenes.append(A.build_scene(sc["air"], sc["sources"], sc["recorders"], p["dh"], p["dt"], p["c0"],
                                    p["pml_layers"]))
    T = max(g["scene"]["steps"] for _, g in runs)
    sim = A.Simulation(scenes, max_steps=T, arithmetic=arith)
    for si, (_, g) in enumerate(runs):
        for i, s in enumerate(g["sources"]):
            ser = np.zeros(T, np.float32)
            ser[:len(s)] = s
            sim.set_source_series(i, ser, scene=si)
    sim.run(T)
    checked = 0
    for si, (name, g) in enumerate(runs):
        got = sim.recorders(scene=si, f64=True)
        want = g["recorders"]
        n = g["scene"]["steps"]
        for r in range(want.shape[1]):
            if np.isnan(want[0, r]) or np.abs(want[:, r]).max() == 0:
                continue
            assert rel_l2(got[:n, r], want[:, r]) < F32_TOL, (name, r)
            checked += 1
    assert checked >= 6
