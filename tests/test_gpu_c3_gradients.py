"""c3 gradient check: the c1 geometry (scene-3 L-shaped room, h = 0.025 m,
1.92 M air cells, 8-cell PML) in FP64, forward + adjoint of the recorder
misfit against a target made with a seeded perturbed source and per-face
damping scales U(0.5, 1.5), checkpoints every 64 steps, checked against
central finite differences: directional derivatives along the source series
and along the six face scales.  512 steps (the gradient check; the full
8000-step c3 run is timed in bench.py)."""
import numpy as np
import pytest

import ard_gb300 as A
from ard_gb300 import configs

pytestmark = pytest.mark.gpu

T = 512


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
    pert = np.zeros_like(series)
    pert[:, :256] = (np.round(rng.standard_normal((nsrc, 256)) * 8) / 64 * k).astype(np.float32)

    def load(s, sc6):
        sim.reset()
        for i in range(nsrc):
            sim.set_source_series(i, s[i])
        sim.set_pml_scale(sc6)

    load(series + pert, scales)
    sim.run(T)
    target = sim.recorders().astype(np.float32)

    def J(s, sc6):
        load(s, sc6)
        sim.run(T)
        return 0.5 * float(np.sum((sim.recorders(f64=True) - target.astype(np.float64)) ** 2))

    load(series, scales)
    g = sim.adjoint(T, target, checkpoint_every=64)
    d = (rng.choice([-1.0, 1.0], size=series.shape) * k / 64).astype(np.float32)
    fd = (J(series + d, scales) - J(series - d, scales)) / 2.0
    ad = float(np.sum(g["grad_source"].astype(np.float64) * d))
    assert abs(ad - fd) <= 1e-3 * abs(fd), (ad, fd)
    ds = np.float32(1.0 / 256) * rng.choice([-1.0, 1.0], size=6).astype(np.float32)
    fds = (J(series, scales + ds) - J(series, scales - ds)) / 2.0
    ads = float(np.sum(g["grad_scale"][0].astype(np.float64) * ds))
    assert abs(ads - fds) <= 1e-3 * abs(fds), (ads, fds)
