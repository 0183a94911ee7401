"""Shared helpers for the tests: golden loading and scene conversion."""
import json
import os

import numpy as np

from conftest import GOLDEN


def load_run(name):
    path = os.path.join(GOLDEN, f"run_{name}.npz")
    if not os.path.exists(path):
        return None
    z = np.load(path, allow_pickle=False)
    scene = json.loads(str(z["scene"]))
    scene["air"] = [tuple(b) for b in scene["air"]]
    scene["sources"] = [tuple(s) for s in scene["sources"]]
    scene["recorders"] = [tuple(r) for r in scene["recorders"]]
    return dict(recorders=z["recorders"], sources=z["sources"], field_sha256=list(z["field_sha256"]),
                scene=scene, setup=str(z["setup"]).splitlines())


def parse_setup(lines):
    """Reference setup dump -> (partitions, boundaries, sources, recorders)."""
    P, B, S, R = [], [], [], []
    for line in lines:
        t = line.split()
        if not t:
            continue
        if t[0] == "P":
            P.append((0 if t[2] == "DCT" else 1, int(t[3])) + tuple(int(v) for v in t[4:10]))
        elif t[0] == "B":
            ab = float.fromhex(t[-1]) if "x" in t[-1] else float(t[-1])
            B.append(tuple(int(v) for v in t[2:11]) + (round(ab, 6),))
        elif t[0] == "S":
            S.append((int(t[1]), int(t[2])))
        elif t[0] == "R":
            R.append((int(t[1]), int(t[2])))
    return P, B, S, R


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))
