"""GPU forms of the reference's post-step products against the oracle's
restatements (oracle/post_oracle.py) and the FP64 C oracle:

  * ard_record_neighbourhoods / ard_read_neighbourhoods / out_<r>.txt
    (Recorder::RecordField, recorder.cpp:40-57): the 10x10x10 cube of every
    step against the FP64 C oracle's field (FP64 context; the history is
    float, so to float rounding), its centre against the point recorder,
    graphs against direct launches bitwise, the text file against the
    recorded values (6 significant digits, as an ostream writes a float);
  * ard_render_slice (simulation.cpp:320-420): the drawn pressure against the
    slices of the partitions' fields (1e-5 of the scene's scale), the pixel
    words bit for bit against the restated colour map of that pressure, the
    uncovered pixels untouched;
  * ard_impulse_response (auralization.m:22-32, t60.m): the FP64 result
    against the numpy restatement to 1e-9, the T60 equal.
"""
import os

import numpy as np
import pytest

import ard_gb300 as A
from oracle import oracle as O
from oracle import post_oracle as P

pytestmark = pytest.mark.gpu

DH, C0 = 0.1, 343.0
DT = float(np.float32(0.5 * DH / (C0 * np.sqrt(3.0))))
AIR = [(0, 0, 0, 20, 20, 16), (20, 4, 0, 12, 12, 16)]
SRC = [(6, 7, 8)]
REC = [(12, 10, 8), (26, 10, 8)]


def series(T):
    return (1e3 * np.exp(-((np.arange(T) - 20.0) ** 2) / 18.0)).astype(np.float32)


def make_sim(T, precision=A.PREC_F32, graphs=True):
    scene = A.build_scene(AIR, SRC, REC, DH, DT, C0, 5)
    sim = A.Simulation(scene, precision=precision, max_steps=T, use_graphs=graphs)
    sim.set_source_series(0, series(T))
    return scene, sim


def local(scene, r):
    x, y, z, part = scene.recorders[r]
    q = scene.partitions[part]
    return part, x - q[2], y - q[3], z - q[4]


def test_neighbourhoods_match_fp64_oracle():
    T, chunk = 96, 32
    scene, sim = make_sim(T, precision=A.PREC_F64)
    sim.record_neighbourhoods(True)
    flat = O.make_flat_scene(AIR, SRC, REC, dict(dh=DH, dt=DT, c0=C0, pml_layers=5))
    ref = O.OracleSim(flat, "f64")
    ref.set_source_series(0, series(T))
    for c in range(T // chunk):
        sim.run(chunk)
        ref.step(chunk)
        cubes = sim.neighbourhoods(t0=(c + 1) * chunk - 1, nt=1)[0]
        for r in range(len(REC)):
            part, x, y, z = local(scene, r)
            want = P.neighbourhood(ref.field(part)[0], x, y, z).reshape(10, 10, 10)
            scale = max(np.abs(want).max(), 1e-30)
            assert np.abs(cubes[r] - want).max() <= 2e-6 * scale, (c, r)


def test_neighbourhood_centre_is_the_recorder_and_graphs_match_direct():
    T = 80
    for prec in (A.PREC_F32, A.PREC_F64):
        runs = []
        for graphs in (True, False):
            _, sim = make_sim(T, precision=prec, graphs=graphs)
            k0 = sim.kernels_per_step
            sim.record_neighbourhoods(True)
            extra = sim.kernels_per_step - k0     # three launches per air group holding recorders
            assert extra in (3, 6)
            sim.run(T)
            cubes = sim.neighbourhoods()
            rec = sim.recorders(f64=True)
            for r in range(len(REC)):
                centre = cubes[:, r, 5, 5, 5].astype(np.float64)
                scale = np.abs(rec[:, r]).max()
                assert scale > 0
                assert np.abs(centre - rec[:, r]).max() <= 1e-5 * scale, (prec, graphs, r)
            runs.append(cubes)
            sim.close()
        assert np.array_equal(runs[0], runs[1]), prec


def test_neighbourhoods_after_reset_and_refusals():
    T = 40
    scene, sim = make_sim(T)
    with pytest.raises(A.ArdError) as e:
        sim.neighbourhoods(nt=1)
    assert e.value.code == 4                      # not recorded
    sim.run(5)
    sim.record_neighbourhoods(True)
    sim.run(10)
    with pytest.raises(A.ArdError) as e:
        sim.neighbourhoods(t0=0, nt=15)           # steps before the recording began
    assert e.value.code == 6
    late = sim.neighbourhoods(t0=5, nt=10)
    sim.reset()
    sim.run(15)
    full = sim.neighbourhoods(t0=0, nt=15)
    assert np.array_equal(full[5:], late)
    # a recorder whose cube leaves its partition (here attached by hand, past
    # Recorder::FindPartition's margin) is refused
    flat = O.make_flat_scene(AIR, SRC, REC, dict(dh=DH, dt=DT, c0=C0, pml_layers=5))
    flat["recorders"] = [(12, 10, 3, 0)]
    sim2 = A.Simulation(A.scene_from_flat(flat), max_steps=8)
    with pytest.raises(A.ArdError) as e:
        sim2.record_neighbourhoods(True)
    assert e.value.code == 1


def test_out_file_matches_recorded_neighbourhoods(tmp_path):
    T = 30
    _, sim = make_sim(T)
    sim.record_neighbourhoods(True)
    sim.run(T)
    sim.write_outputs(str(tmp_path))
    cubes = sim.neighbourhoods()
    for r in range(len(REC)):
        lines = open(os.path.join(tmp_path, f"out_{r}.txt")).read().split("\n")
        assert lines[-1] == "" and len(lines) == T + 1
        for t in (0, 17, T - 1):
            assert lines[t].endswith(" ")
            vals = np.array([float(v) for v in lines[t].split()])
            assert vals.shape == (1000,)
            want = cubes[t, r].ravel().astype(np.float64)
            assert np.allclose(vals, want, rtol=1e-5, atol=1e-30 + 1e-6 * np.abs(want).max())
        assert os.path.exists(os.path.join(tmp_path, f"response_{r}.txt"))


@pytest.mark.parametrize("look_from", [0, 1])
def test_slice_colour_map(look_from):
    import torch
    T = 40
    scene, sim = make_sim(T)
    sim.run(T)
    w, h = sim.slice_size(look_from)
    sentinel = np.uint32(0x12345678)
    pix = torch.full((h, w), int(np.int32(sentinel.view(np.int32))), dtype=torch.int32, device="cuda")
    pres = torch.zeros((h, w), dtype=torch.float32, device="cuda")
    coord = SRC[0][2] if look_from == 0 else SRC[0][0]
    sim.render_slice(look_from, coord, pixels=pix, pressure=pres)
    got_pix = pix.cpu().numpy().view(np.uint32)
    got_p = pres.cpu().numpy()
    parts = scene.partitions
    fields = [sim.field(i) for i in range(len(parts))]
    image = np.full((h, w), sentinel, np.uint32)
    want_pix, want_p = P.render_slice(parts, fields, look_from, coord, image=image)
    covered = want_pix != sentinel
    assert covered.any()
    assert np.all(got_pix[~covered] == sentinel)
    scale = max(np.abs(f).max() for f in fields)
    assert np.abs(got_p - want_p)[covered].max() <= 1e-5 * scale
    # the colour of every drawn pixel is the reference's formula of its pressure, bit for bit
    assert np.array_equal(got_pix[covered], P.slice_colour(got_p[covered]))
    # and differs from the colour of the readout's pressure only where a rounding boundary lies between them
    assert np.mean(got_pix[covered] == want_pix[covered]) > 0.99


def test_impulse_response_matches_restatement():
    T = 600
    _, sim = make_sim(T)
    sim.run(T)
    sr = 1.0 / DT
    for trunc, fcut in ((0, 1500.0), (400, 1000.0)):
        rir, t60 = sim.impulse_response(recorder=0, source=0, truncate=trunc, sample_rate=sr, fcut=fcut)
        want = P.rir(sim.recorders(f64=True)[:, 0], series(T), truncate=trunc, fcut=fcut, sr=sr, order=1024)
        assert np.abs(rir - want).max() <= 1e-9
        rt, slope, stop, overrun = P.t60(want, sr)
        assert t60["t60_ms"] == rt and t60["stop"] == stop and t60["overrun"] == overrun
        assert abs(t60["slope"] - slope) <= 1e-6 * abs(slope)
    with pytest.raises(A.ArdError):
        sim.impulse_response(fcut=0.6 * sr)   # above the Nyquist rate
