"""Profiling driver: build one of the benchmark workloads and run a few
direct-launch steps (no CUDA graphs, so every kernel is a separate launch
for ncu), optionally printing the per-stage device times.

    python ard-simulator_gb300/ard_gb300/profile_run.py CONFIG STEPS [stages] [N_SCENES]
"""
from __future__ import annotations

import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

import ard_gb300 as A  # noqa: E402
from ard_gb300 import configs  # noqa: E402


def main(argv):
    name, n = argv[1], int(argv[2])
    want_stages = len(argv) > 3 and argv[3] == "stages"
    cfg = configs.config(name, steps=max(n, 64))
    scs = cfg["scenes"][: (int(argv[4]) if len(argv) > 4 else 1)]
    scenes = [A.build_scene(sc["air"], sc["sources"], sc["recorders"], cfg["h"], cfg["dt"], cfg["c0"], cfg["pml"])
              for sc in scs]
    sim = A.Simulation(scenes, max_steps=max(n, 64) * 4, use_graphs=False)
    for k, sc in enumerate(scs):
        for i, s in enumerate(sc["series"]):
            sim.set_source_series(i, s[:max(n, 64)], scene=k)
    sim.run(n)
    sim.synchronize()
    if want_stages:
        print(json.dumps({k: round(v * 1000, 1) for k, v in sim.profile(50).items()}))
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv))
