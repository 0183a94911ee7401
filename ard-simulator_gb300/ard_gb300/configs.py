"""Synthetic workloads: the five benchmark scenes, seeded.

All geometry follows the reference's conventions: air partitions as cell
boxes (x, y, z, width, height, depth), 2.5D (every partition spans the same
z range), sources and recorders as cells.  Time step "CFL 0.5" means
dt = 0.5 h / (c sqrt(3)), i.e. c dt / h = 0.289 (the literal c dt / h = 0.5
exceeds the 6th-order PML leapfrog limit of 0.470).

  c0  single 5 m cube at h = 0.05 (100^3 cells), 5-cell PML, Gaussian pulse
      (sigma 3 samples, peak at step 20, amplitude 1e9) at (1, 1, 1) m,
      recorder at (4, 4, 4) m, 2000 steps
  c1  the reference's scene-3 L-shaped room (assets/scene-3.txt) at
      h = 0.025, 8-cell PML, seeded source / 4 recorders, 8000 steps
  c2  512 independent scenes, each a seeded guillotine decomposition into
      2-12 rectangles with sides U(0.5, 4) m snapped to h = 0.05, common
      depth U(2, 3) m, 5-cell PML, 1 source + 4 recorders, 4000 steps
  c3  c1 geometry for forward + adjoint
  c4  40 x 25 m footprint, 12 m deep, 24 seeded partitions at h = 0.04
      (~1.9e8 cells), 10-cell PML, 16 recorders, 20000 steps
  c4one  the largest c4 partition alone (profiling case, 12.4 M cells)
"""
from __future__ import annotations

import numpy as np

C_SOUND = 343.0
SCENE3_METRES = [(0, 0, 0, 3, 3, 2), (0, 3, 0, 2, 1, 2), (3, 0, 0, 1, 2, 2),
                 (4, 0, 0, 1, 1, 2), (0, 4, 0, 1, 1, 2)]


def dt_cfl(h, c=C_SOUND, cfl=0.5):
    return float(np.float32(cfl * h / (c * np.sqrt(3.0))))


def gaussian_pulse(n, peak=20.0, sigma=3.0, amplitude=1e9):
    t = np.arange(n, dtype=np.float64)
    return (amplitude * np.exp(-((t - peak) ** 2) / (2.0 * sigma * sigma))).astype(np.float32)


def metres_to_cells(v, h):
    """(int)(v / h) with the division in float32 (partition.cpp:159-163)."""
    return int(np.float32(np.float32(v) / np.float32(h)))


def pick_points(rng, boxes, n, margin_lo=6, margin_hi=5):
    """Uniform cells in the air, volume-weighted over partitions, with the
    recorder margin of Recorder::FindPartition (x - x0 >= 6, x1 - x >= 5)."""
    ok = [b for b in boxes if min(b[3], b[4], b[5]) >= margin_lo + margin_hi + 1]
    vol = np.array([b[3] * b[4] * b[5] for b in ok], np.float64)
    pts = []
    for _ in range(n):
        b = ok[rng.choice(len(ok), p=vol / vol.sum())]
        pts.append(tuple(int(rng.integers(b[i] + margin_lo, b[i] + b[3 + i] - margin_hi + 1)) for i in range(3)))
    return pts


def config(name, steps=None, seed=1):
    """dict(name, h, c0, dt, pml, steps, scenes=[dict(air, sources, recorders, series)])."""
    if name == "c0":
        h = 0.05
        air = [(0, 0, 0, 100, 100, 100)]
        n = steps or 2000
        sc = dict(air=air, sources=[(20, 20, 20)], recorders=[(80, 80, 80)], series=[gaussian_pulse(n)])
        return dict(name=name, h=h, c0=C_SOUND, dt=dt_cfl(h), pml=5, steps=n, scenes=[sc])
    if name in ("c1", "c3"):
        h = 0.025
        air = [tuple(metres_to_cells(v, h) for v in b) for b in SCENE3_METRES]
        rng = np.random.default_rng(seed)
        src = pick_points(rng, air, 1)
        rec = pick_points(rng, air, 4)
        n = steps or 8000
        sc = dict(air=air, sources=src, recorders=rec, series=[gaussian_pulse(n)])
        return dict(name=name, h=h, c0=C_SOUND, dt=dt_cfl(h), pml=8, steps=n, scenes=[sc])
    if name == "c2":
        h = 0.05
        n = steps or 4000
        rng = np.random.default_rng(seed)
        scenes = [_guillotine_scene(rng, h, n) for _ in range(512)]
        return dict(name=name, h=h, c0=C_SOUND, dt=dt_cfl(h), pml=5, steps=n, scenes=scenes)
    if name == "c4":
        h = 0.04
        n = steps or 20000
        rng = np.random.default_rng(seed)
        W, H, D = metres_to_cells(40, h), metres_to_cells(25, h), metres_to_cells(12, h)
        rects = _split_to(rng, [(0, 0, W, H)], 24, min_side=100)
        air = [(x, y, 0, w, hh, D) for (x, y, w, hh) in rects]
        src = pick_points(rng, air, 1)
        rec = pick_points(rng, air, 16)
        return dict(name=name, h=h, c0=C_SOUND, dt=dt_cfl(h), pml=10, steps=n,
                    scenes=[dict(air=air, sources=src, recorders=rec, series=[gaussian_pulse(n)])])
    if name == "c4one":
        # profiling case: the largest c4 partition alone (232 x 178 x 300 cells at h = 0.04)
        h = 0.04
        n = steps or 200
        air = [(0, 0, 0, 232, 178, 300)]
        sc = dict(air=air, sources=[(40, 50, 150)], recorders=[(180, 120, 100)], series=[gaussian_pulse(n)])
        return dict(name=name, h=h, c0=C_SOUND, dt=dt_cfl(h), pml=10, steps=n, scenes=[sc])
    raise ValueError(name)


def _split_to(rng, rects, count, min_side):
    """Guillotine: split the largest rectangle across its longer side until
    `count` rectangles exist, keeping every side >= min_side cells."""
    rects = list(rects)
    while len(rects) < count:
        rects.sort(key=lambda r: r[2] * r[3])
        x, y, w, hh = rects.pop()
        if w >= hh:
            if w < 2 * min_side:
                rects.append((x, y, w, hh)); break
            cut = int(rng.integers(min_side, w - min_side + 1))
            rects += [(x, y, cut, hh), (x + cut, y, w - cut, hh)]
        else:
            if hh < 2 * min_side:
                rects.append((x, y, w, hh)); break
            cut = int(rng.integers(min_side, hh - min_side + 1))
            rects += [(x, y, w, cut), (x, y + cut, w, hh - cut)]
    return rects


def _guillotine_scene(rng, h, steps):
    """2-12 rectangles, sides in [0.5, 4] m snapped to h, common depth U(2, 3) m."""
    lo, hi = metres_to_cells(0.5, h), metres_to_cells(4.0, h)
    n = int(rng.integers(2, 13))
    while True:
        W = int(rng.integers(2 * lo, 2 * hi + 1))
        H = int(rng.integers(lo, 2 * hi + 1))
        rects = [(0, 0, W, H)]
        # split until n pieces and every side <= hi
        guard = 0
        while (len(rects) < n or max(max(r[2], r[3]) for r in rects) > hi) and guard < 200:
            guard += 1
            rects.sort(key=lambda r: max(r[2], r[3]))
            x, y, w, hh = rects.pop()
            if w >= hh and w >= 2 * lo:
                cut = int(rng.integers(lo, w - lo + 1))
                rects += [(x, y, cut, hh), (x + cut, y, w - cut, hh)]
            elif hh >= 2 * lo:
                cut = int(rng.integers(lo, hh - lo + 1))
                rects += [(x, y, w, cut), (x, y + cut, w, hh - cut)]
            else:
                rects.append((x, y, w, hh))
                break
        if (2 <= len(rects) <= 12 and all(lo <= min(r[2], r[3]) and max(r[2], r[3]) <= hi for r in rects)
                and any(min(r[2], r[3]) >= 12 for r in rects)):
            break
    D = int(rng.integers(metres_to_cells(2.0, h), metres_to_cells(3.0, h) + 1))
    air = [(x, y, 0, w, hh, D) for (x, y, w, hh) in rects]
    src = pick_points(rng, air, 1)
    rec = pick_points(rng, air, 4)
    return dict(air=air, sources=src, recorders=rec, series=[gaussian_pulse(steps)])
