"""ORACLE / TEST INFRASTRUCTURE ONLY -- the checker, never the product.

ctypes front end of liboracle.so (ard_oracle.c in float and double) plus a
helper that drives the headless reference build.  Only tests/, the smoke
check and bench.py's CPU-baseline leg import this module.

Scenes are passed as "flat scenes": a dict with
  params      dict(dh, dt, c0, pml_layers, pml_R, modal_damping)
  partitions  [(kind, pml_type, x, y, z, w, h, d)]
  boundaries  [(type, a, b, xs, xe, ys, ye, zs, ze, absorption)]
  sources     [(x, y, z, partition)]
  recorders   [(x, y, z, partition)]
which is field for field the C struct ard_scene of include/ard_gb300.h.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import tempfile

import numpy as np

from . import build_oracle, scene_oracle


class _Partition(C.Structure):
    _fields_ = [("kind", C.c_int32), ("pml_type", C.c_int32),
                ("x_start", C.c_int32), ("y_start", C.c_int32), ("z_start", C.c_int32),
                ("width", C.c_int32), ("height", C.c_int32), ("depth", C.c_int32)]


class _Boundary(C.Structure):
    _fields_ = [("type", C.c_int32), ("a", C.c_int32), ("b", C.c_int32),
                ("x_start", C.c_int32), ("x_end", C.c_int32), ("y_start", C.c_int32),
                ("y_end", C.c_int32), ("z_start", C.c_int32), ("z_end", C.c_int32),
                ("absorption", C.c_float)]


class _Point(C.Structure):
    _fields_ = [("x", C.c_int32), ("y", C.c_int32), ("z", C.c_int32), ("partition", C.c_int32)]


class _Scene(C.Structure):
    _fields_ = [("dh", C.c_float), ("dt", C.c_float), ("c0", C.c_float),
                ("pml_layers", C.c_int32), ("pml_R", C.c_float), ("modal_damping", C.c_float),
                ("n_partitions", C.c_int32), ("partitions", C.POINTER(_Partition)),
                ("n_boundaries", C.c_int32), ("boundaries", C.POINTER(_Boundary)),
                ("n_sources", C.c_int32), ("sources", C.POINTER(_Point)),
                ("n_recorders", C.c_int32), ("recorders", C.POINTER(_Point))]


def _array(ctype, rows):
    arr = (ctype * max(1, len(rows)))()
    for i, r in enumerate(rows):
        arr[i] = ctype(*r)
    return arr


def pack_scene(flat):
    """Flat scene -> (ard_scene, keep-alive list)."""
    p = flat["params"]
    parts = _array(_Partition, flat["partitions"])
    bnds = _array(_Boundary, flat["boundaries"])
    srcs = _array(_Point, flat["sources"])
    recs = _array(_Point, flat["recorders"])
    sc = _Scene(p["dh"], p["dt"], p["c0"], p["pml_layers"], p.get("pml_R", 1e-5),
                p.get("modal_damping", 0.999),
                len(flat["partitions"]), parts, len(flat["boundaries"]), bnds,
                len(flat["sources"]), srcs, len(flat["recorders"]), recs)
    return sc, [parts, bnds, srcs, recs]


def flat_from_setup(built, params, sources, recorders):
    """scene_oracle.build_scene output -> flat scene."""
    parts = [(q.kind, q.pml_type, q.x, q.y, q.z, q.w, q.h, q.d) for q in built["partitions"]]
    bnds = [(b.type, b.a, b.b, b.xs, b.xe, b.ys, b.ye, b.zs, b.ze, b.absorption)
            for b in built["boundaries"]]
    srcs = [(x, y, z, pi) for (x, y, z), pi in zip(sources, built["source_part"])]
    recs = [(x, y, z, pi) for (x, y, z), pi in zip(recorders, built["recorder_part"])]
    return dict(params=dict(params), partitions=parts, boundaries=bnds, sources=srcs,
                recorders=recs)


def make_flat_scene(air_boxes, sources, recorders, params):
    built = scene_oracle.build_scene(air_boxes, sources, recorders, params["pml_layers"],
                                     params.get("absorption", 1.0))
    return flat_from_setup(built, params, sources, recorders)


_LIB = None


def lib():
    global _LIB
    if _LIB is None:
        path = build_oracle.build_oracle()
        L = C.CDLL(path)
        for sfx in ("_f32", "_f64"):
            getattr(L, "oracle_create" + sfx).restype = C.c_void_p
            getattr(L, "oracle_create" + sfx).argtypes = [C.POINTER(_Scene)]
            getattr(L, "oracle_destroy" + sfx).argtypes = [C.c_void_p]
            getattr(L, "oracle_set_source_series" + sfx).argtypes = [
                C.c_void_p, C.c_int, C.POINTER(C.c_float), C.c_long]
            getattr(L, "oracle_set_pml_scale" + sfx).argtypes = [C.c_void_p, C.POINTER(C.c_double)]
            getattr(L, "oracle_set_initial_pressure" + sfx).argtypes = [
                C.c_void_p, C.c_int, C.POINTER(C.c_double)]
            getattr(L, "oracle_step" + sfx).argtypes = [C.c_void_p, C.c_long]
            getattr(L, "oracle_time_step" + sfx).restype = C.c_long
            getattr(L, "oracle_time_step" + sfx).argtypes = [C.c_void_p]
            getattr(L, "oracle_read_recorders" + sfx).argtypes = [C.c_void_p, C.POINTER(C.c_double)]
            getattr(L, "oracle_read_field" + sfx).argtypes = [
                C.c_void_p, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        _LIB = L
    return _LIB


def _dptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class OracleSim:
    """The C restatement on one flat scene; precision 'f32' or 'f64'."""

    def __init__(self, flat, precision="f32"):
        self.flat = flat
        self.sfx = "_" + precision
        self.L = lib()
        sc, self._keep = pack_scene(flat)
        self._sc = sc
        self.h = getattr(self.L, "oracle_create" + self.sfx)(C.byref(sc))

    def _f(self, name):
        return getattr(self.L, name + self.sfx)

    def close(self):
        if self.h:
            self._f("oracle_destroy")(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_source_series(self, i, series):
        s = np.ascontiguousarray(series, dtype=np.float32)
        self._f("oracle_set_source_series")(self.h, i, s.ctypes.data_as(C.POINTER(C.c_float)), s.size)

    def set_pml_scale(self, scale6):
        s = np.ascontiguousarray(scale6, dtype=np.float64)
        self._f("oracle_set_pml_scale")(self.h, _dptr(s))

    def set_initial_pressure(self, part, p0):
        a = np.ascontiguousarray(p0, dtype=np.float64).ravel()
        self._f("oracle_set_initial_pressure")(self.h, part, _dptr(a))

    def step(self, n):
        self._f("oracle_step")(self.h, n)

    @property
    def time_step(self):
        return self._f("oracle_time_step")(self.h)

    def recorders(self):
        t = self.time_step
        out = np.zeros((t, len(self.flat["recorders"])), np.float64)
        if out.size:
            self._f("oracle_read_recorders")(self.h, _dptr(out))
        return out

    def field(self, part):
        q = self.flat["partitions"][part]
        shape = (q[7], q[6], q[5])
        p = np.zeros(shape, np.float64)
        f = np.zeros(shape, np.float64)
        self._f("oracle_read_field")(self.h, part, _dptr(p), _dptr(f))
        return p, f


# ---------------------------------------------------------------------------
# headless reference build driver (only where the reference sources exist)
# ---------------------------------------------------------------------------

def reference_available():
    return os.path.isdir(build_oracle.REFDIR)


def run_reference(air_boxes, sources, recorders, params, steps, series=None,
                  mode="parity", field_steps=(), threads=1, workdir=None):
    """Runs oracle/_ref/ard_ref.  sources: [(x, y, z)], with `series` a list of
    float32 arrays (one per source) or None for the reference GaussianSource.
    Returns dict(setup=[lines], recorders=[T, R] float32, sources=[S, T]
    float32 (the values injected), fields={step: float32 array}, info=dict)."""
    binpath = build_oracle.build_reference()
    if binpath is None:
        raise RuntimeError("reference sources not present")
    own = workdir is None
    wd = tempfile.mkdtemp(prefix="ardref_") if own else workdir
    out = os.path.join(wd, "out")
    lines = [f"dh {float(np.float32(params['dh'])).hex()}",
             f"dt {float(np.float32(params['dt'])).hex()}",
             f"c0 {float(np.float32(params['c0'])).hex()}",
             f"absorption {float(np.float32(params.get('absorption', 1.0))).hex()}",
             f"pml_layers {params['pml_layers']}", f"steps {steps}", f"mode {mode}",
             f"out {out}", f"partitions {len(air_boxes)}"]
    lines += [" ".join(str(v) for v in b) for b in air_boxes]
    lines.append(f"sources {len(sources)}")
    for i, (x, y, z) in enumerate(sources):
        if series is None:
            lines.append(f"{x} {y} {z} gaussian")
        else:
            s = np.asarray(series[i], np.float32)
            lines.append(f"{x} {y} {z} series {s.size} " + " ".join(float(v).hex() for v in s))
    lines.append(f"recorders {len(recorders)}")
    lines += [f"{x} {y} {z}" for (x, y, z) in recorders]
    lines.append(f"fields {len(field_steps)} " + " ".join(str(s) for s in field_steps))
    cfg = os.path.join(wd, "config.txt")
    with open(cfg, "w") as f:
        f.write("\n".join(lines) + "\n")
    env = dict(os.environ, OMP_NUM_THREADS=str(threads))
    res = subprocess.run([binpath, cfg], cwd=wd, env=env, capture_output=True, text=True, check=True)
    import json
    info = json.loads(res.stdout.strip().splitlines()[-1])
    with open(os.path.join(out, "setup.txt")) as f:
        setup = f.read().splitlines()
    rec = np.fromfile(os.path.join(out, "recorders.f32"), np.float32)
    rec = rec.reshape(steps, len(recorders)) if recorders else np.zeros((steps, 0), np.float32)
    src = np.fromfile(os.path.join(out, "sources.f32"), np.float32).reshape(len(sources), steps)
    fields = {}
    for s in field_steps:
        with open(os.path.join(out, f"fields_{s}.f32"), "rb") as f:
            fields[s] = np.frombuffer(f.read(), np.float32)
    if own:
        import shutil
        shutil.rmtree(wd, ignore_errors=True)
    return dict(setup=setup, recorders=rec, sources=src, fields=fields, info=info)
