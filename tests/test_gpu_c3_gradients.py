"""c3 gradient check: the c1 geometry (scene-3 L-shaped room, h = 0.025 m,
1.92 M air cells, 8-cell PML) in FP64, forward + adjoint of the recorder
misfit against a target made with the c3 perturbation (the source series
plus 1024 samples of seeded noise band-limited at 2 kHz, then zeros) and
per-face damping scales U(0.5, 1.5), checkpoints every 64 steps, checked
against central finite differences: directional derivatives along the
source series, along the initial pressure of the largest air partition and
along the six face scales.  1280 steps (past the 1024 samples of noise; the
full 8000-step c3 run is timed in bench.py).

J is quadratic in the series and in the initial pressure, so their central
differences are exact up to rounding when the perturbed inputs are exactly
representable in the float32 the ABI takes: the series and the directions
are dyadic.  The face-scale derivative is a smooth nonlinear one (step
2^-8)."""
import numpy as np
import pytest

import ard_gb300 as A
from ard_gb300 import configs

pytestmark = pytest.mark.gpu

T = 1280


def band_limited_noise(rng, n_src, S, dt, amp):
    noise = rng.standard_normal((n_src, S))
    spec = np.fft.rfft(noise, axis=1)
    spec[:, np.fft.rfftfreq(S, d=dt) > 2000.0] = 0     # 2 kHz band limit
    x = np.fft.irfft(spec, n=S, axis=1)
    pert = 0.1 * amp * x / (np.abs(x).max() + 1e-30)
    pert[:, 1024:] = 0                                  # 1024 samples of noise, then zeros
    return pert.astype(np.float32)


def test_c3_gradients_match_central_differences():
    cfg = configs.config("c3", steps=T)
    sc = cfg["scenes"][0]
    scene = A.build_scene(sc["air"], sc["sources"], sc["recorders"], cfg["h"], cfg["dt"], cfg["c0"], cfg["pml"])
    sim = A.Simulation(scene, precision=A.PREC_F64, max_steps=T, adjoint=True)
    rng = np.random.default_rng(3)
    nsrc = len(sc["sources"])
    # dyadic series on a 2^-6 grid of the pulse amplitude: exact perturbations in FP32
    amp = float(np.abs(sc["series"][0][:T]).max())
    k = 2.0 ** np.floor(np.log2(amp))
    series = np.stack([np.round(np.asarray(s[:T], np.float64) / k * 64) / 64 * k for s in sc["series"]]).astype(np.float32)
    scales = np.float32(np.round(rng.uniform(0.5, 1.5, 6) * 256) / 256)
    pert = band_limited_noise(rng, nsrc, T, cfg["dt"], amp)
    part = int(np.argmax([p[5] * p[6] * p[7] if p[0] == A.PART_DCT else 0 for p in scene.partitions]))
    q = scene.partitions[part]
    shape = (q[7], q[6], q[5])

    def load(s, sc6, p0=None):
        sim.reset()
        for i in range(nsrc):
            sim.set_source_series(i, s[i])
        sim.set_pml_scale(sc6)
        if p0 is not None:
            sim.set_initial_pressure(part, p0)

    load(series + pert, scales)
    sim.run(T)
    target = sim.recorders().astype(np.float32)

    def J(s, sc6, p0=None):
        load(s, sc6, p0)
        sim.run(T)
        return 0.5 * float(np.sum((sim.recorders(f64=True) - target.astype(np.float64)) ** 2))

    load(series, scales)
    g = sim.adjoint(T, target, checkpoint_every=64)
    gp0 = sim.initial_pressure_grad(part).astype(np.float64)
    # source series
    d = (rng.choice([-1.0, 1.0], size=series.shape) * k / 64).astype(np.float32)
    fd = (J(series + d, scales) - J(series - d, scales)) / 2.0
    ad = float(np.sum(g["grad_source"].astype(np.float64) * d))
    assert abs(ad - fd) <= 1e-3 * abs(fd), (ad, fd)
    # initial pressure of the largest air partition (the adjoint ran from rest)
    rec_amp = float(np.abs(target).max())
    kp = 2.0 ** np.floor(np.log2(rec_amp))
    dp = (rng.choice([-1.0, 1.0], size=shape) * kp).astype(np.float32)
    fdp = (J(series, scales, dp) - J(series, scales, -dp)) / 2.0
    adp = float(np.sum(gp0 * dp))
    assert abs(fdp) > 0
    assert abs(adp - fdp) <= 1e-3 * abs(fdp), (adp, fdp)
    # face scales
    ds = np.float32(1.0 / 256) * rng.choice([-1.0, 1.0], size=6).astype(np.float32)
    fds = (J(series, scales + ds) - J(series, scales - ds)) / 2.0
    ads = float(np.sum(g["grad_scale"][0].astype(np.float64) * ds))
    assert abs(ads - fds) <= 1e-3 * abs(fds), (ads, fds)
