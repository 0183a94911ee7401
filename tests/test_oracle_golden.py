"""The oracle is pinned to the reference: the float build of the C
restatement reproduces the headless reference build bit for bit (recorder
samples and the sha256 of every partition's pressure and force field), and
the product's Gaussian source matches GaussianSource::SampleValue exactly."""
import hashlib

import numpy as np
import pytest
import scipy.fft as sf

import ard_gb300 as A
from helpers import load_run, rel_l2
from oracle import oracle as O


def _oracle_run(g, precision="f32"):
    sc = g["scene"]
    flat = O.make_flat_scene(sc["air"], sc["sources"], sc["recorders"], sc["params"])
    sim = O.OracleSim(flat, precision)
    for i, s in enumerate(g["sources"]):
        sim.set_source_series(i, s)
    sim.step(sc["steps"])
    return flat, sim


@pytest.mark.parametrize("name", ["multi4", "scene2_gauss", "quirk_run", "c0_40"])
def test_oracle_matches_reference_bit_for_bit(name):
    g = load_run(name)
    assert g is not None
    flat, sim = _oracle_run(g)
    rec = sim.recorders().astype(np.float32)
    want = g["recorders"]
    ok = ~np.isnan(want)
    assert np.array_equal(rec[ok], want[ok])
    for i, hsh in enumerate(g["field_sha256"]):
        p, f = sim.field(i)
        got = hashlib.sha256(np.concatenate([p.ravel(), f.ravel()]).astype(np.float32).tobytes()).hexdigest()
        assert got == hsh, f"partition {i}"


def test_fp64_oracle_close_to_reference():
    g = load_run("multi4")
    _, sim = _oracle_run(g, "f64")
    rec = sim.recorders()
    for r in range(rec.shape[1]):
        assert rel_l2(rec[:, r], g["recorders"][:, r]) < 1e-4


def test_gaussian_source_matches_reference():
    g = load_run("scene2_gauss")
    p = g["scene"]["params"]
    s = A.gaussian_series(p["c0"], p["dt"], p["dh"], g["scene"]["steps"])
    assert np.array_equal(s, g["sources"][0])


@pytest.mark.parametrize("n", [1, 2, 3, 7, 10, 13, 37, 80, 100, 120])
def test_oracle_dct_matches_scipy(n):
    import ctypes as C
    from oracle import build_oracle
    lib = C.CDLL(build_oracle.build_oracle())
    lib.dctfft_3d_double.argtypes = [C.c_int] * 4 + [C.c_void_p] * 2
    rng = np.random.default_rng(n)
    a = rng.standard_normal((3, 2, n))
    o = np.empty_like(a)
    lib.dctfft_3d_double(3, 2, n, 10, a.ctypes.data, o.ctypes.data)
    np.testing.assert_allclose(o, sf.dctn(a, type=2), rtol=1e-12, atol=1e-12)
    lib.dctfft_3d_double(3, 2, n, 1, a.ctypes.data, o.ctypes.data)
    np.testing.assert_allclose(o, sf.dctn(a, type=3), rtol=1e-12, atol=1e-12)


def test_literal_cfl_half_diverges():
    """c dt / h = 0.5 (the literal "CFL 0.5") makes the reference algorithm
    blow up: the 6th-order leapfrog with the PML damping terms is stable at
    c dt / h = 0.43 (the reference's own dh = 0.1 m, dt = 1/8000 s) and
    diverges at 0.45, so the library refuses scenes above 0.44."""
    h, c = 0.1, 343.0

    def run(cfl):
        dt = float(np.float32(cfl * h / c))
        flat = O.make_flat_scene([(0, 0, 0, 12, 12, 12)], [(6, 6, 6)], [(6, 6, 6)],
                                 dict(dh=h, dt=dt, c0=c, pml_layers=5))
        sim = O.OracleSim(flat, "f64")
        sim.set_source_series(0, np.r_[np.float32(1.0), np.zeros(1999, np.float32)])
        sim.step(1500)
        return flat, max(np.abs(sim.field(i)[0]).max() for i in range(len(flat["partitions"])))

    flat, blown = run(0.5)
    assert not np.isfinite(blown) or blown > 1e6
    _, ok = run(0.43)
    assert np.isfinite(ok) and ok < 1.0
    for cfl in (0.5, 0.45):
        flat, _ = O.make_flat_scene([(0, 0, 0, 12, 12, 12)], [(6, 6, 6)], [(6, 6, 6)],
                                    dict(dh=h, dt=float(np.float32(cfl * h / c)), c0=c, pml_layers=5)), None
        with pytest.raises(A.ArdError) as e:
            A.Simulation(A.scene_from_flat(flat))
        assert e.value.code == 5  # ARD_ERR_UNSTABLE, checked before any device work
