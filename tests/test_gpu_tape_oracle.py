"""The hand-written adjoint (ard_adjoint, FP64 GPU context) against the FP64
autograd tape of oracle/tape_oracle.py on the same scene and inputs:
gradients with respect to the source series, the initial pressure and the
six PML face scales, to 1e-8 relative.  Also drives the torch.autograd
bridge (ard_gb300.autograd.RecorderMisfit)."""
import numpy as np
import pytest

import ard_gb300 as A
from ard_gb300.autograd import RecorderMisfit
from oracle import oracle as O
from oracle.tape_oracle import TapeOracle

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

DH, C0 = 0.1, 343.0
DT = float(np.float32(0.5 * DH / (C0 * np.sqrt(3.0))))
AIR = [(0, 0, 0, 16, 14, 12), (16, 1, 0, 12, 12, 12)]
SOURCES = [(4, 5, 5), (20, 6, 4)]
RECORDERS = [(8, 6, 6), (10, 8, 7), (22, 7, 6)]
T = 40


def rel(a, b):
    a = np.asarray(a, np.float64); b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.fixture(scope="module")
def case():
    rng = np.random.default_rng(5)
    series = rng.standard_normal((len(SOURCES), T)).astype(np.float32)
    p0 = rng.standard_normal((12, 14, 16)).astype(np.float32)
    scale = np.array([1.0, 0.75, 1.25, 1.0, 0.5, 1.5], np.float32)
    flat = O.make_flat_scene(AIR, SOURCES, RECORDERS, dict(dh=DH, dt=DT, c0=C0, pml_layers=5))
    tape = TapeOracle(flat)
    s_t = torch.tensor(series, dtype=torch.float64, requires_grad=True)
    p_t = torch.tensor(p0, dtype=torch.float64, requires_grad=True)
    z_t = torch.tensor(scale, dtype=torch.float64, requires_grad=True)
    rec = tape.run(s_t, T, p0={0: p_t}, scale6=z_t)
    target = (0.5 * rec.detach().numpy()[::-1]).astype(np.float32)   # what the library takes
    J = 0.5 * ((rec - torch.tensor(target, dtype=torch.float64)) ** 2).sum()
    J.backward()
    scene = A.build_scene(AIR, SOURCES, RECORDERS, DH, DT, C0, 5)
    sim = A.Simulation(scene, precision=A.PREC_F64, max_steps=T, adjoint=True)
    return dict(series=series, p0=p0, scale=scale, target=target, J=float(J.detach()),
                gs=s_t.grad.numpy(), gp=p_t.grad.numpy(), gz=z_t.grad.numpy(), sim=sim)


def test_adjoint_matches_fp64_tape(case):
    sim = case["sim"]
    sim.reset()
    for i in range(len(SOURCES)):
        sim.set_source_series(i, case["series"][i])
    sim.set_initial_pressure(0, case["p0"])
    sim.set_pml_scale(case["scale"])
    g = sim.adjoint(T, case["target"], checkpoint_every=8)
    assert abs(g["loss"][0] - case["J"]) <= 1e-6 * case["J"]       # the loss comes back as float
    assert rel(g["grad_source"], case["gs"]) < 1e-7                # float output: its rounding
    assert rel(sim.initial_pressure_grad(0), case["gp"]) < 1e-6    # read back as float
    assert rel(g["grad_scale"][0], case["gz"]) < 1e-6


def test_autograd_bridge(case):
    sim = case["sim"]
    s = torch.tensor(case["series"], dtype=torch.float64, requires_grad=True)
    z = torch.tensor(case["scale"], dtype=torch.float64, requires_grad=True)
    J = RecorderMisfit.apply(s, z, sim, T, case["target"])
    (2.0 * J).backward()
    # no initial pressure here: compare with a tape run without it
    flat = O.make_flat_scene(AIR, SOURCES, RECORDERS, dict(dh=DH, dt=DT, c0=C0, pml_layers=5))
    s_t = torch.tensor(case["series"], dtype=torch.float64, requires_grad=True)
    z_t = torch.tensor(case["scale"], dtype=torch.float64, requires_grad=True)
    rec = TapeOracle(flat).run(s_t, T, scale6=z_t)
    Jt = 0.5 * ((rec - torch.tensor(case["target"], dtype=torch.float64)) ** 2).sum()
    (2.0 * Jt).backward()
    assert rel(s.grad.numpy(), s_t.grad.numpy()) < 1e-6
    assert rel(z.grad.numpy(), z_t.grad.numpy()) < 1e-6
