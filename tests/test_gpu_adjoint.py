"""Adjoint of the ARD step (ard_adjoint): gradients of the recorder misfit
J = 0.5 sum (rec - target)^2 against central finite differences of J in the
FP64 context.

J is quadratic in the source series and in the initial pressure, so a
central difference with an exactly representable step (dyadic inputs, step
1/16 or 1/64) equals the directional derivative up to rounding of J itself:
tolerance 1e-6 relative.  J is smooth but not quadratic in the PML face
scales: step 2^-8, truncation O(step^2), tolerance 2e-5 relative.  The FP32
gradients are compared with the FP64 ones at 2e-3 relative L2."""
import numpy as np
import pytest

import ard_gb300 as A

pytestmark = pytest.mark.gpu

T_STEPS = 80
DH, C0, PML = 0.1, 343.0, 5
DT = 0.5 * DH / (C0 * np.sqrt(3.0))
AIR = [(0, 0, 0, 16, 14, 12), (16, 1, 0, 12, 12, 12)]   # two air partitions, 12 PML slabs, 12 interfaces
SOURCES = [(4, 5, 5), (20, 6, 4)]
RECORDERS = [(8, 6, 6), (10, 8, 7), (22, 7, 6)]


def dyadic(rng, shape, bits=10):
    """Values k / 2^bits in [-1, 1]: sums with small powers of two stay exact in FP32."""
    return (rng.integers(-(1 << bits), (1 << bits) + 1, size=shape) / float(1 << bits)).astype(np.float32)


class Problem:
    """Seeded inputs; with p0=False the partitions start at rest, so the
    recorders carry the source-driven signal alone (about dt^2 times the
    series amplitude, far below an initial pressure's) and the target is
    drawn on that signal's scale."""

    def __init__(self, precision=A.PREC_F64, arithmetic=A.ARITH_ACCURATE, seed=0, p0=True):
        rng = np.random.default_rng(seed)
        self.scene = A.build_scene(AIR, SOURCES, RECORDERS, DH, DT, C0, PML)
        self.sim = A.Simulation(self.scene, precision=precision, max_steps=T_STEPS, arithmetic=arithmetic,
                                adjoint=True)
        self.series = dyadic(rng, (len(SOURCES), T_STEPS))
        parts = self.scene.partitions
        self.p0 = [dyadic(rng, (q[7], q[6], q[5])) * (1 if p0 else 0) for q in parts[:len(AIR)]]
        self.scale = np.ones(6, np.float32)
        self.target = np.zeros((T_STEPS, len(RECORDERS)), np.float32)
        self.prepare()
        self.sim.run(T_STEPS)
        rms = float(np.sqrt(np.mean(self.sim.recorders(f64=True) ** 2)))
        self.target = (0.5 * rms * rng.standard_normal((T_STEPS, len(RECORDERS)))).astype(np.float32)

    def prepare(self, series=None, p0=None, scale=None):
        sim = self.sim
        sim.reset()
        s = self.series if series is None else series
        for i in range(len(SOURCES)):
            sim.set_source_series(i, s[i])
        for k, p in enumerate(self.p0 if p0 is None else p0):
            sim.set_initial_pressure(k, p)
        sim.set_pml_scale(self.scale if scale is None else scale)

    def J(self, **kw):
        self.prepare(**kw)
        self.sim.run(T_STEPS)
        rec = self.sim.recorders(f64=True)
        return 0.5 * float(np.sum((rec - self.target.astype(np.float64)) ** 2))

    def grads(self, checkpoint_every=0, want_scale=True, **kw):
        self.prepare(**kw)
        g = self.sim.adjoint(T_STEPS, self.target, checkpoint_every=checkpoint_every, want_scale=want_scale)
        g["p0"] = [self.sim.initial_pressure_grad(k) for k in range(len(AIR))]
        return g


@pytest.fixture(scope="module", params=[A.ARITH_ACCURATE, A.ARITH_REFERENCE], ids=["accurate", "reference"])
def problem(request):
    pr = Problem(arithmetic=request.param)
    pr.g = pr.grads(checkpoint_every=16)
    return pr


@pytest.fixture(scope="module", params=[A.ARITH_ACCURATE, A.ARITH_REFERENCE], ids=["accurate", "reference"])
def src_problem(request):
    pr = Problem(arithmetic=request.param, p0=False)
    pr.g = pr.grads(checkpoint_every=16)
    return pr


def test_loss_matches_forward(problem):
    assert abs(problem.g["loss"][0] - problem.J()) <= 1e-6 * problem.J()


def test_source_series_gradient(src_problem):
    problem = src_problem
    rng = np.random.default_rng(1)
    d = rng.choice([-1.0, 1.0], size=problem.series.shape).astype(np.float32)
    eps = 1.0 / 16
    fd = (problem.J(series=problem.series + eps * d) - problem.J(series=problem.series - eps * d)) / (2 * eps)
    ad = float(np.sum(problem.g["grad_source"].astype(np.float64) * d))
    assert abs(ad - fd) <= 1e-6 * abs(fd), (ad, fd)
    # one source alone, one step alone: single entries of the gradient
    for (q, t) in [(0, 3), (1, 40)]:
        e = np.zeros_like(problem.series)
        e[q, t] = 1.0
        fd1 = (problem.J(series=problem.series + eps * e) - problem.J(series=problem.series - eps * e)) / (2 * eps)
        assert abs(problem.g["grad_source"][q, t] - fd1) <= 1e-6 * abs(fd) + 1e-6 * abs(fd1), (q, t)


def test_initial_pressure_gradient(problem):
    rng = np.random.default_rng(2)
    eps = 1.0 / 64
    for k in range(len(AIR)):
        d = rng.choice([-1.0, 1.0], size=problem.p0[k].shape).astype(np.float32)
        plus = [p.copy() for p in problem.p0]
        minus = [p.copy() for p in problem.p0]
        plus[k] += eps * d
        minus[k] -= eps * d
        fd = (problem.J(p0=plus) - problem.J(p0=minus)) / (2 * eps)
        ad = float(np.sum(problem.g["p0"][k].astype(np.float64) * d))
        assert abs(ad - fd) <= 1e-6 * abs(fd), (k, ad, fd)


def test_pml_scale_gradient(problem):
    eps = 1.0 / 256
    g = problem.g["grad_scale"][0]
    for f in range(6):
        sp = problem.scale.copy(); sp[f] += eps
        sm = problem.scale.copy(); sm[f] -= eps
        fd = (problem.J(scale=sp) - problem.J(scale=sm)) / (2 * eps)
        assert abs(g[f] - fd) <= 2e-5 * np.abs(g).max(), (f, g[f], fd)


def test_checkpoint_interval_does_not_change_gradients(problem, monkeypatch):
    for K in (0, 7, T_STEPS):   # 0: the whole PML history kept in one forward run; else PML replay
        g = problem.grads(checkpoint_every=K)
        assert ("whole PML history" if K == 0 else "PML replay") in problem.sim.layout
        np.testing.assert_allclose(g["grad_scale"], problem.g["grad_scale"], rtol=1e-10, atol=0)
        np.testing.assert_allclose(g["grad_source"], problem.g["grad_source"], rtol=1e-10, atol=1e-30)
    # the segment-recompute path (used where the replay's forcing record does not fit)
    monkeypatch.setenv("ARD_ADJOINT_RECOMPUTE", "1")
    g = problem.grads(checkpoint_every=9)
    assert "segment recompute" in problem.sim.layout
    np.testing.assert_allclose(g["grad_scale"], problem.g["grad_scale"], rtol=1e-10, atol=0)
    np.testing.assert_allclose(g["grad_source"], problem.g["grad_source"], rtol=1e-10, atol=1e-30)
    # the hybrid: the first two of nine segments recomputed, the rest replayed
    monkeypatch.setenv("ARD_ADJOINT_RECOMPUTE", "3")
    g = problem.grads(checkpoint_every=9)
    assert "hybrid" in problem.sim.layout and "first 2 of 9" in problem.sim.layout
    np.testing.assert_allclose(g["grad_scale"], problem.g["grad_scale"], rtol=1e-10, atol=0)
    np.testing.assert_allclose(g["grad_source"], problem.g["grad_source"], rtol=1e-10, atol=1e-30)
    for k in range(len(AIR)):
        np.testing.assert_allclose(g["p0"][k], problem.g["p0"][k], rtol=1e-10, atol=1e-30)
    monkeypatch.delenv("ARD_ADJOINT_RECOMPUTE")
    # without the damping gradient nothing is checkpointed: the other gradients stay
    g = problem.grads(want_scale=False)
    assert g["grad_scale"] is None
    np.testing.assert_allclose(g["grad_source"], problem.g["grad_source"], rtol=1e-10, atol=1e-30)
    for k in range(len(AIR)):
        np.testing.assert_allclose(g["p0"][k], problem.g["p0"][k], rtol=1e-10, atol=1e-30)


def test_adjoint_leaves_the_forward_after_step_T():
    pr = Problem(seed=3)
    pr.prepare()
    pr.sim.run(T_STEPS)
    want = pr.sim.recorders(f64=True)
    field = pr.sim.field(0)
    pr.grads(checkpoint_every=9)
    assert pr.sim.time_step == T_STEPS
    np.testing.assert_array_equal(pr.sim.recorders(f64=True), want)
    np.testing.assert_array_equal(pr.sim.field(0), field)


def test_fp32_gradients_follow_fp64():
    g64 = Problem(precision=A.PREC_F64, seed=4).grads(checkpoint_every=20)
    g32 = Problem(precision=A.PREC_F32, seed=4).grads(checkpoint_every=20)

    def rel(a, b):
        a = np.asarray(a, np.float64); b = np.asarray(b, np.float64)
        return np.linalg.norm(a - b) / np.linalg.norm(b)

    assert rel(g32["grad_source"], g64["grad_source"]) < 2e-3
    assert rel(g32["grad_scale"], g64["grad_scale"]) < 2e-3
    for k in range(len(AIR)):
        assert rel(g32["p0"][k], g64["p0"][k]) < 2e-3


def test_fp32_tensor_core_adjoint(monkeypatch):
    """FP32 with the face transforms forced onto the two-pass form: the
    forward's and the adjoint's face passes run on the tensor cores (split
    TF32).  Gradients within 1e-4 relative L2 of the same FP32 problem on the
    fused CUDA-core face kernel, and within the FP32 bar of FP64."""
    def rel(a, b):
        a = np.asarray(a, np.float64); b = np.asarray(b, np.float64)
        return np.linalg.norm(a - b) / np.linalg.norm(b)

    g64 = Problem(precision=A.PREC_F64, seed=5).grads(checkpoint_every=20)
    fused = Problem(precision=A.PREC_F32, seed=5)
    assert "faces fused" in fused.sim.layout
    gf = fused.grads(checkpoint_every=20)
    monkeypatch.setenv("ARD_FACE_TWO_PASS", "1")
    mma = Problem(precision=A.PREC_F32, seed=5)
    assert "faces tensor-core" in mma.sim.layout
    gm = mma.grads(checkpoint_every=20)
    for key in ("grad_source", "grad_scale"):
        assert rel(gm[key], gf[key]) < 1e-4, key
        assert rel(gm[key], g64[key]) < 2e-3, key
    for k in range(len(AIR)):
        assert rel(gm["p0"][k], gf["p0"][k]) < 1e-4, k
        assert rel(gm["p0"][k], g64["p0"][k]) < 2e-3, k


def test_adjoint_errors():
    scene = A.build_scene(AIR, SOURCES, RECORDERS, DH, DT, C0, PML)
    plain = A.Simulation(scene, precision=A.PREC_F64, max_steps=T_STEPS)
    tgt = np.zeros((T_STEPS, len(RECORDERS)), np.float32)
    with pytest.raises(A.ArdError):
        plain.adjoint(T_STEPS, tgt)                   # context without options.adjoint
    sim = A.Simulation(scene, precision=A.PREC_F64, max_steps=T_STEPS, adjoint=True)
    with pytest.raises(A.ArdError):
        sim.initial_pressure_grad(0)                  # no adjoint run yet
    with pytest.raises(A.ArdError):
        sim.adjoint(T_STEPS + 1, np.zeros((T_STEPS + 1, len(RECORDERS)), np.float32))   # beyond max_steps
    sim.run(1)
    with pytest.raises(A.ArdError):
        sim.adjoint(T_STEPS, tgt)                     # not at step 0


def test_adjoint_through_gemm_face_transforms():
    """FP64 with faces of 139-141 rows (more than the fused face kernel's
    128, not multiples of 4): the face transforms (and their transposes) take
    the two-pass GEMM path with scalar staging; source-series and face-scale
    gradients against central differences."""
    dh, c0 = 0.1, 343.0
    dt = 0.5 * dh / (c0 * np.sqrt(3.0))
    air, srcs, recs = [(0, 0, 0, 141, 139, 15)], [(30, 40, 7)], [(60, 55, 7), (20, 80, 6)]
    T = 60
    scene = A.build_scene(air, srcs, recs, dh, dt, c0, 5)
    sim = A.Simulation(scene, precision=A.PREC_F64, max_steps=T, adjoint=True)
    assert "gemm" in sim.layout
    rng = np.random.default_rng(11)
    series = dyadic(rng, (1, T))
    scale = np.ones(6, np.float32)

    def run(s, sc):
        sim.reset()
        sim.set_source_series(0, s[0])
        sim.set_pml_scale(sc)

    run(series, scale)
    sim.run(T)
    rms = float(np.sqrt(np.mean(sim.recorders(f64=True) ** 2)))
    target = (0.5 * rms * rng.standard_normal((T, len(recs)))).astype(np.float32)

    def J(s, sc):
        run(s, sc)
        sim.run(T)
        return 0.5 * float(np.sum((sim.recorders(f64=True) - target.astype(np.float64)) ** 2))

    run(series, scale)
    g = sim.adjoint(T, target, checkpoint_every=16)
    d = rng.choice([-1.0, 1.0], size=series.shape).astype(np.float32)
    eps = 1.0 / 16
    fd = (J(series + eps * d, scale) - J(series - eps * d, scale)) / (2 * eps)
    ad = float(np.sum(g["grad_source"].astype(np.float64) * d))
    assert abs(ad - fd) <= 1e-6 * abs(fd), (ad, fd)
    e = 1.0 / 256
    for f in (0, 5):
        sp = scale.copy(); sp[f] += e
        sm = scale.copy(); sm[f] -= e
        fds = (J(series, sp) - J(series, sm)) / (2 * e)
        assert abs(g["grad_scale"][0][f] - fds) <= 2e-5 * np.abs(g["grad_scale"][0]).max(), f
