"""ORACLE / TEST INFRASTRUCTURE ONLY -- the checker, never the product.

Pure-Python restatement of the reference's scene setup, used to check the
product's C++ scene builder.  It follows, in ARD-simulator-190113/:

* ``Boundary::FindBoundary`` (boundary.cpp:289-334): two partitions sharing an
  x face (x overlap == 0, y overlap > 0) get an X interface six cells wide
  centred on the shared face, spanning the y overlap and ``a``'s z range;
  likewise for y.
* ``Partition::AddBoundary`` (partition.cpp:96-143): marks the face cells an
  X/Y interface covers as not free, on every z slice.
* ``Simulation::Simulation`` (simulation.cpp:14-294): pairwise interface
  discovery (i < j), source attachment (half-open box test), then for every
  air partition in order: left, right, top, bottom PML runs found on z-slice
  0 of the free-border maps (with the reference's end-of-row quirk), then the
  always-present front and back PMLs; each PML is appended to the partition
  list and its interface to the boundary list.
* ``Recorder::FindPartition`` (recorder.cpp:26-38): first air partition with
  the 5-cell margin.
* ``Partition::ImportPartitions`` / ``SoundSource::ImportSources`` /
  ``Recorder::ImportRecorders``: integer metres divided by dh in float32 and
  truncated.

Pinned against the headless reference build's setup dump (tests/golden).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

DCT, PML = 0, 1
P_LEFT, P_RIGHT, P_TOP, P_BOTTOM, P_FRONT, P_BACK = range(6)
X_BOUNDARY, Y_BOUNDARY, Z_BOUNDARY = range(3)


@dataclass
class Part:
    kind: int
    pml_type: int
    x: int
    y: int
    z: int
    w: int
    h: int
    d: int
    # free-border maps [depth][height] / [depth][width] / ...
    left: list = field(default_factory=list)
    right: list = field(default_factory=list)
    top: list = field(default_factory=list)
    bottom: list = field(default_factory=list)

    @property
    def xe(self):
        return self.x + self.w

    @property
    def ye(self):
        return self.y + self.h

    @property
    def ze(self):
        return self.z + self.d


@dataclass
class Bound:
    type: int
    a: int
    b: int
    xs: int
    xe: int
    ys: int
    ye: int
    zs: int
    ze: int
    absorption: float


def _new_air(x, y, z, w, h, d):
    p = Part(DCT, -1, x, y, z, w, h, d)
    p.left = [[True] * h for _ in range(d)]
    p.right = [[True] * h for _ in range(d)]
    p.top = [[True] * w for _ in range(d)]
    p.bottom = [[True] * w for _ in range(d)]
    return p


def find_boundary(parts, ia, ib, absorp):
    a, b = parts[ia], parts[ib]
    x_ov = min(a.xe, b.xe) - max(a.x, b.x)
    y_ov = min(a.ye, b.ye) - max(a.y, b.y)
    zs, ze = a.z, a.z + a.d
    if x_ov == 0 and y_ov > 0:
        xs = a.xe - 3 if a.xe == b.x else b.xe - 3
        ys = a.y + max(0, b.y - a.y)
        return Bound(X_BOUNDARY, ia, ib, xs, xs + 6, ys, ys + y_ov, zs, ze, absorp)
    if y_ov == 0 and x_ov > 0:
        xs = a.x + max(0, b.x - a.x)
        ys = a.ye - 3 if a.ye == b.y else b.ye - 3
        return Bound(Y_BOUNDARY, ia, ib, xs, xs + x_ov, ys, ys + 6, zs, ze, absorp)
    return None


def add_boundary(p: Part, bd: Bound):
    if bd.type == X_BOUNDARY:
        target = p.left if (bd.xs < p.x and bd.xe > p.x) else p.right
        for i in range(p.d):
            for j in range(bd.ys, bd.ye):
                target[i][j - p.y] = False
    elif bd.type == Y_BOUNDARY:
        target = p.top if (bd.ys < p.y and bd.ye > p.y) else p.bottom
        for i in range(p.d):
            for j in range(bd.xs, bd.xe):
                target[i][j - p.x] = False


def _runs(free_row, n):
    """PML runs along one face (simulation.cpp:54-212): yields (start, length)."""
    start = end = 0
    started = False
    for i in range(n):
        if started:
            end += 1
            if free_row[i] and i != n - 1:
                continue
            elif start != end:
                if i != n - 1:
                    end -= 1
                yield start, end - start + 1
                started = False
        elif free_row[i]:
            start = end = i
            started = True


def build_scene(air_boxes, sources, recorders, pml_layers, absorption=1.0):
    """air_boxes: [(x, y, z, w, h, d)] cells; sources/recorders: [(x, y, z)].

    Returns dict(partitions=[...], boundaries=[...], source_part=[...],
    recorder_part=[...]) in the reference's list orders.
    """
    parts = [_new_air(*b) for b in air_boxes]
    bounds = []
    n_air = len(parts)
    for i in range(n_air):
        for j in range(i + 1, n_air):
            bd = find_boundary(parts, i, j, 1.0)
            if bd is not None:
                bounds.append(bd)
                add_boundary(parts[i], bd)
                add_boundary(parts[j], bd)
    source_part = []
    for (sx, sy, sz) in sources:
        hit = -1
        for i in range(n_air):
            p = parts[i]
            if p.x <= sx < p.xe and p.y <= sy < p.ye and p.z <= sz < p.ze:
                hit = i  # the reference attaches to every match; boxes do not overlap
                break
        source_part.append(hit)
    L = pml_layers
    for c in range(n_air):
        p = parts[c]
        for (start, n) in _runs(p.left[0], p.h):
            parts.append(Part(PML, P_LEFT, p.x - L, p.y + start, p.z, L, n, p.d))
            bounds.append(find_boundary(parts, len(parts) - 1, c, absorption))
        for (start, n) in _runs(p.right[0], p.h):
            parts.append(Part(PML, P_RIGHT, p.xe, p.y + start, p.z, L, n, p.d))
            bounds.append(find_boundary(parts, len(parts) - 1, c, absorption))
        for (start, n) in _runs(p.top[0], p.w):
            parts.append(Part(PML, P_TOP, p.x + start, p.y - L, p.z, n, L, p.d))
            bounds.append(find_boundary(parts, len(parts) - 1, c, absorption))
        for (start, n) in _runs(p.bottom[0], p.w):
            parts.append(Part(PML, P_BOTTOM, p.x + start, p.ye, p.z, n, L, p.d))
            bounds.append(find_boundary(parts, len(parts) - 1, c, absorption))
        parts.append(Part(PML, P_FRONT, p.x, p.y, p.z - L, p.w, p.h, L))
        bounds.append(Bound(Z_BOUNDARY, len(parts) - 1, c, p.x, p.xe, p.y, p.ye,
                            p.z - 3, p.z + 3, absorption))
        parts.append(Part(PML, P_BACK, p.x, p.y, p.ze, p.w, p.h, L))
        bounds.append(Bound(Z_BOUNDARY, len(parts) - 1, c, p.x, p.xe, p.y, p.ye,
                            p.ze - 3, p.ze + 3, absorption))
    recorder_part = []
    for (rx, ry, rz) in recorders:
        hit = -1
        for i in range(n_air):
            p = parts[i]
            if (p.x < rx - 5 and p.xe > rx + 4 and p.y < ry - 5 and p.ye > ry + 4
                    and p.z < rz - 5 and p.ze > rz + 4):
                hit = i
                break
        recorder_part.append(hit)
    return dict(partitions=parts, boundaries=bounds, source_part=source_part,
                recorder_part=recorder_part)


def metres_to_cells(values, dh):
    """(int)(value / dh) with the division in float32, as the importers do."""
    dh32 = np.float32(dh)
    return [int(np.float32(np.float32(v) / dh32)) for v in values]


def import_text(path, dh, group):
    """Read integer-metre rows of `group` ints and convert to cells."""
    rows = []
    with open(path) as f:
        toks = f.read().split()
    vals = [int(t) for t in toks]
    for i in range(0, len(vals) - len(vals) % group, group):
        rows.append(tuple(metres_to_cells(vals[i:i + group], dh)))
    return rows


def setup_lines(scene):
    """Canonical text form of the reference driver's setup.txt records
    (absorption written as a decimal float)."""
    out = []
    for i, p in enumerate(scene["partitions"]):
        out.append(f"P {i} {'DCT' if p.kind == DCT else 'PML'} {p.pml_type} "
                   f"{p.x} {p.y} {p.z} {p.w} {p.h} {p.d}")
    for i, b in enumerate(scene["boundaries"]):
        out.append(f"B {i} {b.type} {b.a} {b.b} {b.xs} {b.xe} {b.ys} {b.ye} {b.zs} {b.ze} "
                   f"{float(np.float32(b.absorption))!r}")
    return out
