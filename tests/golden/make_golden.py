"""Generates the committed golden fixtures from the reference itself.

Runs the headless reference build (oracle/ref_build: the reference's own
sources, compiled in place with SDL / FFTW / VkFFT stand-ins) on small
scenes and on the c0 / c1 benchmark scenes, and writes:

  setup_<name>.txt   the reference's partition / boundary / source /
                     recorder lists after Simulation's constructor
  run_<name>.npz     recorder samples (float32 [T, R]), injected source
                     values (float32 [S, T]), sha256 of every partition's
                     pressure and force field after the last step (when
                     recorded), and the scene definition

Usage (needs the reference sources on this machine):
    python tests/golden/make_golden.py [--long] [--c2]
--long also produces the full-length c0 (2000 steps) and c1 (8000 steps)
recorder series, which take tens of minutes on the host; --c2 the runs of
three c2 scenes (300-400 steps, a few minutes).
"""
from __future__ import annotations

import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(REPO, "ard-simulator_gb300"))

from oracle import build_oracle  # noqa: E402
from oracle import oracle as O  # noqa: E402
from oracle import scene_oracle as SO  # noqa: E402
from ard_gb300 import configs as K  # noqa: E402

ASSETS = os.path.join(build_oracle.REFDIR, "assets")   # the reference's scene files


def params_for(h, c=343.0, pml=5):
    return dict(dh=float(np.float32(h)), dt=K.dt_cfl(h, c), c0=float(np.float32(c)), pml_layers=pml)


def metre_boxes(path, h):
    return SO.import_text(path, h, 6)


def write_setup(name, air, src, rec, params):
    res = O.run_reference(air, src, rec, params, steps=0)
    with open(os.path.join(HERE, f"setup_{name}.txt"), "w") as f:
        f.write("\n".join(res["setup"]) + "\n")


def run_and_store(name, air, src, rec, params, steps, series, fields=True, threads=1):
    field_steps = (steps - 1,) if fields else ()
    res = O.run_reference(air, src, rec, params, steps, series=series, mode="parity",
                          field_steps=field_steps, threads=threads)
    hashes = []
    if fields:
        flat = O.make_flat_scene(air, src, rec, params)
        buf = res["fields"][steps - 1]
        off = 0
        for q in flat["partitions"]:
            n = q[5] * q[6] * q[7]
            hashes.append(hashlib.sha256(buf[off:off + 2 * n].tobytes()).hexdigest())
            off += 2 * n
    scene = dict(air=air, sources=src, recorders=rec, params=params, steps=steps,
                 series="gaussian" if series is None else "given")
    np.savez_compressed(os.path.join(HERE, f"run_{name}.npz"), recorders=res["recorders"],
                        sources=res["sources"], field_sha256=np.array(hashes),
                        scene=np.array(json.dumps(scene)), setup=np.array("\n".join(res["setup"])))
    print(name, res["info"], flush=True)
    return res


def main(long_runs=False, c2_runs=False):
    # --- setup fixtures: the reference's own scene files and synthetic ones ---
    for fname, h in (("scene-1.txt", 0.1), ("scene-2.txt", 0.1), ("scene-3.txt", 0.1),
                     ("scene-3.txt", 0.025), ("hall.txt", 0.2)):
        air = metre_boxes(os.path.join(ASSETS, fname), h)
        name = fname.replace(".txt", "").replace("-", "") + f"_h{h}"
        write_setup(name, air, [], [], params_for(h, pml=8 if h == 0.025 else 5))
    # end-of-row PML quirk: a neighbour covering only the last row of a face,
    # and one starting on the last index
    write_setup("quirk_lastrow", [(0, 0, 0, 20, 20, 12), (20, 19, 0, 10, 10, 12), (-10, 0, 0, 10, 1, 12)][:2],
                [], [], params_for(0.1))
    write_setup("quirk_tjunction", [(0, 0, 0, 30, 20, 12), (30, 5, 0, 12, 10, 12), (10, 20, 0, 12, 12, 12)],
                [], [], params_for(0.1))
    c2 = K.config("c2", steps=16)
    for i in range(3):
        sc = c2["scenes"][i]
        write_setup(f"c2scene{i}", sc["air"], sc["sources"], sc["recorders"], params_for(0.05))

    # --- short runs, fields hashed (bit-exact targets for the float oracle) ---
    T = 80
    air4 = [(0, 0, 0, 20, 20, 20), (10, 20, 0, 10, 10, 20), (20, 10, 0, 10, 30, 20), (30, 20, 0, 10, 20, 20)]
    src4, rec4 = [(5, 5, 5), (25, 30, 8)], [(12, 12, 12), (14, 8, 9)]
    ser4 = [(1e3 * np.exp(-((np.arange(T) - 20.0 - 5 * i) ** 2) / 18.0)).astype(np.float32) for i in range(2)]
    run_and_store("multi4", air4, src4, rec4, params_for(0.1), T, ser4)
    air2 = metre_boxes(os.path.join(ASSETS, "scene-2.txt"), 0.1)
    run_and_store("scene2_gauss", air2, [(5, 5, 5)], [(12, 12, 12)], params_for(0.1), 100, None)
    run_and_store("quirk_run", [(0, 0, 0, 20, 20, 12), (20, 19, 0, 10, 10, 12)], [(4, 4, 6)], [(8, 8, 6)],
                  params_for(0.1), 60, [K.gaussian_pulse(60, amplitude=1e3)])
    c0 = K.config("c0", steps=40)
    sc = c0["scenes"][0]
    run_and_store("c0_40", sc["air"], sc["sources"], sc["recorders"], params_for(0.05), 40, sc["series"],
                  fields=True, threads=8)
    if c2_runs:
        c2_golden_runs()
    if long_runs:
        c0 = K.config("c0")
        sc = c0["scenes"][0]
        run_and_store("c0_full", sc["air"], sc["sources"], sc["recorders"], params_for(0.05), c0["steps"],
                      sc["series"], fields=False, threads=8)
        c1 = K.config("c1")
        sc = c1["scenes"][0]
        run_and_store("c1_full", sc["air"], sc["sources"], sc["recorders"], params_for(0.025, pml=8),
                      c1["steps"], sc["series"], fields=False, threads=8)


# c2 scenes (seeded guillotine decompositions, h = 0.05 m, cell units) run by
# the reference for a few hundred steps: the batched GPU context is checked
# against these scene by scene
C2_RUNS = ((0, 300), (1, 400), (3, 400))


def c2_golden_runs():
    c2 = K.config("c2", steps=max(t for _, t in C2_RUNS))
    for i, steps in C2_RUNS:
        sc = c2["scenes"][i]
        run_and_store(f"c2scene{i}", sc["air"], sc["sources"], sc["recorders"], params_for(0.05), steps,
                      [s[:steps] for s in sc["series"]], fields=False, threads=1)


if __name__ == "__main__":
    main(long_runs="--long" in sys.argv, c2_runs="--c2" in sys.argv)
