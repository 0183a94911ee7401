"""Scene setup (interfaces, PML runs, attachment) against the reference.

The golden setup dumps come from the reference's own Simulation constructor
(tests/golden/make_golden.py).  Both the product's C++ builder
(ard_scene_build / ard_scene_import) and the oracle's Python restatement
must reproduce them exactly, list order included.
"""
import glob
import os

import numpy as np
import pytest

import ard_gb300 as A
from ard_gb300 import configs as K
from conftest import GOLDEN
from helpers import parse_setup
from oracle import scene_oracle as SO

SCENE_FILES = {  # the reference's assets/*.txt partition lists (integer metres)
    "scene1": [(0, 0, 0, 10, 10, 10)],
    "scene2": [(0, 0, 0, 2, 2, 2), (1, 2, 0, 1, 1, 2), (2, 1, 0, 1, 3, 2), (3, 2, 0, 1, 2, 2)],
    "scene3": K.SCENE3_METRES,
    "hall": [(0, 0, 0, 30, 10, 10), (2, 10, 0, 26, 10, 10), (5, 20, 0, 20, 10, 10)],
}
CASES = {
    "scene1_h0.1": ("scene1", 0.1, 5), "scene2_h0.1": ("scene2", 0.1, 5), "scene3_h0.1": ("scene3", 0.1, 5),
    "scene3_h0.025": ("scene3", 0.025, 8), "hall_h0.2": ("hall", 0.2, 5),
}


def _cells(boxes, h):
    return [tuple(SO.metres_to_cells(b, h)) for b in boxes]


def _product(air, src, rec, h, pml):
    sc = A.build_scene(air, src, rec, float(np.float32(h)), K.dt_cfl(h), 343.0, pml)
    P = [tuple(p) for p in sc.partitions]
    B = [tuple(b[:9]) + (round(b[9], 6),) for b in sc.boundaries]
    return sc, P, B


def _golden(name):
    with open(os.path.join(GOLDEN, f"setup_{name}.txt")) as f:
        return parse_setup(f.read().splitlines())


@pytest.mark.parametrize("name", sorted(CASES))
def test_reference_scene_files(name, tmp_path):
    key, h, pml = CASES[name]
    air = _cells(SCENE_FILES[key], h)
    P, B, _, _ = _golden(name)
    _, Pp, Bp = _product(air, [], [], h, pml)
    assert Pp == P
    assert Bp == B
    built = SO.build_scene(air, [], [], pml)
    Po = [(q.kind, q.pml_type, q.x, q.y, q.z, q.w, q.h, q.d) for q in built["partitions"]]
    Bo = [(b.type, b.a, b.b, b.xs, b.xe, b.ys, b.ye, b.zs, b.ze, round(b.absorption, 6)) for b in built["boundaries"]]
    assert Po == P and Bo == B
    # the text importer (integer metres / dh in float, truncated) gives the same scene
    parts = tmp_path / "p.txt"
    parts.write_text("\n".join(" ".join(str(v) for v in b) for b in SCENE_FILES[key]) + "\n\n")
    srcs = tmp_path / "s.txt"
    srcs.write_text("")
    sc = A.import_scene(str(parts), str(srcs), None, float(np.float32(h)), K.dt_cfl(h), 343.0, pml)
    assert [tuple(p) for p in sc.partitions] == P


@pytest.mark.parametrize("name", ["quirk_lastrow", "quirk_tjunction", "c2scene0", "c2scene1", "c2scene2"])
def test_synthetic_scenes(name):
    P, B, S, R = _golden(name)
    air = [p[2:] for p in P if p[0] == 0]
    if name.startswith("c2scene"):
        sc = K.config("c2", steps=16)["scenes"][int(name[-1])]
        src, rec = sc["sources"], sc["recorders"]
        h, pml = 0.05, 5
    else:
        src, rec, h, pml = [], [], 0.1, 5
    scene, Pp, Bp = _product(air, src, rec, h, pml)
    assert Pp == P
    assert Bp == B
    # source attachment and recorder partitions as the reference resolved them
    assert sorted((s[3], i) for i, s in enumerate(scene.sources)) == sorted(S)
    assert [(i, r[3]) for i, r in enumerate(scene.recorders)] == R


def test_end_of_row_quirk_is_reproduced():
    """A neighbour covering only the last row: the right PML over-extends onto it."""
    P, _, _, _ = _golden("quirk_lastrow")
    right = [p for p in P if p[0] == 1 and p[1] == 1 and p[2] == 20 and p[5] == 5]
    assert any(p[6] == 20 for p in right)  # 20 rows although row 19 is shared


def test_builder_rejects_bad_scenes():
    h, dt, c = 0.1, K.dt_cfl(0.1), 343.0
    with pytest.raises(A.ArdError, match="recorder"):
        A.build_scene([(0, 0, 0, 20, 20, 20)], [(5, 5, 5)], [(2, 2, 2)], h, dt, c, 5)
    with pytest.raises(A.ArdError, match="below 6"):
        A.build_scene([(0, 0, 0, 5, 20, 20)], [], [], h, dt, c, 5)
    with pytest.raises(A.ArdError, match="overlap"):
        A.build_scene([(0, 0, 0, 20, 20, 20), (10, 10, 0, 20, 20, 20)], [], [], h, dt, c, 5)
    with pytest.raises(A.ArdError, match="pml_layers"):
        A.build_scene([(0, 0, 0, 20, 20, 20)], [], [], h, dt, c, 3)


def test_all_setup_goldens_are_covered():
    names = {os.path.basename(p)[6:-4] for p in glob.glob(os.path.join(GOLDEN, "setup_*.txt"))}
    covered = set(CASES) | {"quirk_lastrow", "quirk_tjunction", "c2scene0", "c2scene1", "c2scene2"}
    assert names <= covered
