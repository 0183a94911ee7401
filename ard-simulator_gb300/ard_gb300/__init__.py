"""GB300 ARD time step: Python front end of libard_gb300.so.

Mirrors the reference's host interface (ARD-simulator-190113/):

* ``import_scene`` / ``build_scene`` -- ``Partition::ImportPartitions``,
  ``SoundSource::ImportSources``, ``Recorder::ImportRecorders`` and the
  ``Simulation`` constructor's interface / PML generation
  (simulation.cpp:14-294), done by the library's C++ scene builder.
* ``Simulation`` -- ``Simulation::Update`` (simulation.cpp:300-318) on the
  GPU: ``Update()`` advances one step and returns the pre-increment step index
  as the reference does; ``run(n)`` advances n steps; ``recorders()`` returns
  what ``Recorder::RecordField`` would sample each step.

Every call goes through the C ABI in include/ard_gb300.h.  There is no CPU
fallback: loading fails loudly when the library is missing, and stepping
fails with ARD_ERR_NOGPU when no sm_103a device is present.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "libard_gb300.so")

ARD_OK = 0
ERRORS = {1: "ARD_ERR_INVALID", 2: "ARD_ERR_CUDA", 3: "ARD_ERR_OOM", 4: "ARD_ERR_STATE",
          5: "ARD_ERR_UNSTABLE", 6: "ARD_ERR_RANGE", 7: "ARD_ERR_NOGPU"}
PART_DCT, PART_PML = 0, 1
PML_LEFT, PML_RIGHT, PML_TOP, PML_BOTTOM, PML_FRONT, PML_BACK = range(6)
BOUNDARY_X, BOUNDARY_Y, BOUNDARY_Z = range(3)
PREC_F32, PREC_F64 = 0, 1
ARITH_ACCURATE, ARITH_REFERENCE = 0, 1


class ArdError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class Partition(C.Structure):
    _fields_ = [("kind", C.c_int32), ("pml_type", C.c_int32),
                ("x_start", C.c_int32), ("y_start", C.c_int32), ("z_start", C.c_int32),
                ("width", C.c_int32), ("height", C.c_int32), ("depth", C.c_int32)]


class Boundary(C.Structure):
    _fields_ = [("type", C.c_int32), ("a", C.c_int32), ("b", C.c_int32),
                ("x_start", C.c_int32), ("x_end", C.c_int32), ("y_start", C.c_int32),
                ("y_end", C.c_int32), ("z_start", C.c_int32), ("z_end", C.c_int32),
                ("absorption", C.c_float)]


class Point(C.Structure):
    _fields_ = [("x", C.c_int32), ("y", C.c_int32), ("z", C.c_int32), ("partition", C.c_int32)]


class SceneDesc(C.Structure):
    _fields_ = [("dh", C.c_float), ("dt", C.c_float), ("c0", C.c_float),
                ("pml_layers", C.c_int32), ("pml_R", C.c_float), ("modal_damping", C.c_float),
                ("n_partitions", C.c_int32), ("partitions", C.POINTER(Partition)),
                ("n_boundaries", C.c_int32), ("boundaries", C.POINTER(Boundary)),
                ("n_sources", C.c_int32), ("sources", C.POINTER(Point)),
                ("n_recorders", C.c_int32), ("recorders", C.POINTER(Point))]


class SceneParams(C.Structure):
    _fields_ = [("dh", C.c_float), ("dt", C.c_float), ("c0", C.c_float), ("pml_layers", C.c_int32),
                ("absorption", C.c_float), ("pml_R", C.c_float), ("modal_damping", C.c_float)]


class Options(C.Structure):
    _fields_ = [("precision", C.c_int32), ("max_steps", C.c_int64), ("use_graphs", C.c_int32),
                ("device", C.c_int32), ("autotune", C.c_int32), ("arithmetic", C.c_int32),
                ("adjoint", C.c_int32)]


# Every exported symbol with its ctypes signature (checked against the header by the tests).
SIGNATURES = {
    "ard_abi_version": (C.c_int, []),
    "ard_scene_build": (C.c_int, [C.POINTER(SceneParams), C.c_int32, C.POINTER(C.c_int32), C.c_int32,
                                  C.POINTER(C.c_int32), C.c_int32, C.POINTER(C.c_int32), C.POINTER(C.c_void_p)]),
    "ard_scene_import": (C.c_int, [C.POINTER(SceneParams), C.c_char_p, C.c_char_p, C.c_char_p,
                                   C.POINTER(C.c_void_p)]),
    "ard_scene_get": (C.POINTER(SceneDesc), [C.c_void_p]),
    "ard_scene_free": (None, [C.c_void_p]),
    "ard_scene_last_error": (C.c_char_p, []),
    "ard_gaussian_series": (C.c_int, [C.c_float, C.c_float, C.c_float, C.c_int64, C.POINTER(C.c_float)]),
    "ard_create": (C.c_int, [C.POINTER(SceneDesc), C.c_int32, C.POINTER(Options), C.POINTER(C.c_void_p)]),
    "ard_destroy": (C.c_int, [C.c_void_p]),
    "ard_set_source_series": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.POINTER(C.c_float), C.c_int64]),
    "ard_set_source_samples": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_int64, C.c_int64,
                                         C.POINTER(C.c_float)]),
    "ard_set_initial_pressure": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.POINTER(C.c_float)]),
    "ard_set_pml_scale": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_float)]),
    "ard_reset": (C.c_int, [C.c_void_p]),
    "ard_step": (C.c_int, [C.c_void_p, C.c_int64, C.c_void_p]),
    "ard_synchronize": (C.c_int, [C.c_void_p]),
    "ard_time_step": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64)]),
    "ard_read_recorders": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_float), C.c_int64, C.c_int64]),
    "ard_read_recorders_f64": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_double), C.c_int64, C.c_int64]),
    "ard_read_field": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.POINTER(C.c_float)]),
    "ard_read_field_noalloc": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.POINTER(C.c_float), C.c_void_p]),
    "ard_adjoint": (C.c_int, [C.c_void_p, C.c_int64, C.POINTER(C.c_float), C.c_int32, C.POINTER(C.c_float),
                              C.POINTER(C.c_float), C.POINTER(C.c_float)]),
    "ard_read_initial_pressure_grad": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.POINTER(C.c_float)]),
    "ard_kernels_per_step": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32)]),
    "ard_write_outputs": (C.c_int, [C.c_void_p, C.c_int32, C.c_char_p, C.c_int64]),
    "ard_record_neighbourhoods": (C.c_int, [C.c_void_p, C.c_int32]),
    "ard_read_neighbourhoods": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_float), C.c_int64, C.c_int64]),
    "ard_slice_size": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    "ard_render_slice": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_float, C.c_void_p,
                                   C.c_void_p]),
    "ard_impulse_response": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_int64, C.c_int64,
                                       C.c_double, C.c_double, C.c_int32, C.POINTER(C.c_double),
                                       C.POINTER(C.c_double)]),
    "ard_describe": (C.c_int, [C.c_void_p, C.c_char_p, C.c_int64]),
    "ard_profile_steps": (C.c_int, [C.c_void_p, C.c_int64, C.c_void_p, C.POINTER(C.c_float), C.c_int32]),
    "ard_last_error": (C.c_int, [C.c_void_p, C.c_char_p, C.c_int64]),
}

_lib = None


def lib():
    """Load libard_gb300.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: run __graft_entry__.build() (nvcc, sm_103a)")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _fptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def _err(ctx=None):
    buf = C.create_string_buffer(2048)
    lib().ard_last_error(ctx, buf, len(buf))
    return buf.value.decode()


def _check(rc, ctx=None):
    if rc != ARD_OK:
        raise ArdError(rc, _err(ctx))


def gaussian_series(c0, dt, dh, n):
    """GaussianSource::SampleValue(t) for t < n (gaussian_source.cpp:16-20)."""
    out = np.zeros(n, np.float32)
    rc = lib().ard_gaussian_series(c0, dt, dh, n, _fptr(out))
    if rc:
        raise ArdError(rc, lib().ard_scene_last_error().decode())
    return out


class Scene:
    """A flattened scene (the reference's Simulation after construction)."""

    def __init__(self, handle=None, desc=None, keep=None):
        self._h = handle
        self._keep = keep
        self.desc = desc if desc is not None else lib().ard_scene_get(handle).contents

    def __del__(self):
        if getattr(self, "_h", None):
            lib().ard_scene_free(self._h)
            self._h = None

    @property
    def partitions(self):
        d = self.desc
        return [tuple(getattr(d.partitions[i], f) for f, _ in Partition._fields_) for i in range(d.n_partitions)]

    @property
    def boundaries(self):
        d = self.desc
        return [tuple(getattr(d.boundaries[i], f) for f, _ in Boundary._fields_) for i in range(d.n_boundaries)]

    @property
    def sources(self):
        d = self.desc
        return [tuple(getattr(d.sources[i], f) for f, _ in Point._fields_) for i in range(d.n_sources)]

    @property
    def recorders(self):
        d = self.desc
        return [tuple(getattr(d.recorders[i], f) for f, _ in Point._fields_) for i in range(d.n_recorders)]

    @property
    def air_cells(self):
        return sum(p[5] * p[6] * p[7] for p in self.partitions if p[0] == PART_DCT)

    @property
    def pml_cells(self):
        return sum(p[5] * p[6] * p[7] for p in self.partitions if p[0] == PART_PML)

    @property
    def face_cells(self):
        """Interface face cells (each reads 6 and writes 6 values per step)."""
        n = 0
        for b in self.boundaries:
            t, xs, xe, ys, ye, zs, ze = b[0], b[3], b[4], b[5], b[6], b[7], b[8]
            if t == 0:
                n += max(0, ye - ys) * max(0, ze - zs)
            elif t == 1:
                n += max(0, xe - xs) * max(0, ze - zs)
            else:
                n += max(0, xe - xs) * max(0, ye - ys)
        return n


def _params(dh, dt, c0, pml_layers, absorption=1.0, pml_R=0.0, modal_damping=0.0):
    return SceneParams(dh, dt, c0, pml_layers, absorption, pml_R, modal_damping)


def build_scene(air_boxes, sources, recorders, dh, dt, c0, pml_layers, absorption=1.0):
    """Scene from air partitions in cells [(x, y, z, w, h, d)], sources and
    recorders as cells [(x, y, z)], by the reference's setup rules."""
    p = _params(dh, dt, c0, pml_layers, absorption)
    boxes = np.ascontiguousarray(np.asarray(air_boxes, np.int32).reshape(-1, 6))
    src = np.ascontiguousarray(np.asarray(sources, np.int32).reshape(-1, 3))
    rec = np.ascontiguousarray(np.asarray(recorders, np.int32).reshape(-1, 3))
    h = C.c_void_p()
    ip = lambda a: a.ctypes.data_as(C.POINTER(C.c_int32))
    rc = lib().ard_scene_build(C.byref(p), len(boxes), ip(boxes), len(src), ip(src), len(rec), ip(rec), C.byref(h))
    if rc:
        raise ArdError(rc, lib().ard_scene_last_error().decode())
    return Scene(h)


def import_scene(partitions_path, sources_path, recorders_path, dh, dt, c0, pml_layers, absorption=1.0):
    """Scene from the reference's integer-metre text files (README.md:13-37)."""
    p = _params(dh, dt, c0, pml_layers, absorption)
    h = C.c_void_p()
    rc = lib().ard_scene_import(C.byref(p), partitions_path.encode(), sources_path.encode(),
                                recorders_path.encode() if recorders_path else None, C.byref(h))
    if rc:
        raise ArdError(rc, lib().ard_scene_last_error().decode())
    return Scene(h)


def scene_from_flat(flat):
    """Scene from plain lists: dict(params, partitions, boundaries, sources,
    recorders) with the ard_scene field order."""
    p = flat["params"]

    def arr(t, rows):
        a = (t * max(1, len(rows)))()
        for i, r in enumerate(rows):
            a[i] = t(*r)
        return a

    parts = arr(Partition, flat["partitions"])
    bnds = arr(Boundary, flat["boundaries"])
    srcs = arr(Point, flat["sources"])
    recs = arr(Point, flat["recorders"])
    d = SceneDesc(p["dh"], p["dt"], p["c0"], p["pml_layers"], p.get("pml_R", 1e-5), p.get("modal_damping", 0.999),
                  len(flat["partitions"]), parts, len(flat["boundaries"]), bnds,
                  len(flat["sources"]), srcs, len(flat["recorders"]), recs)
    return Scene(None, d, keep=[parts, bnds, srcs, recs])


class Simulation:
    """Context over one or many scenes (many = batched mode)."""

    def __init__(self, scenes, precision=PREC_F32, max_steps=4096, use_graphs=True, device=0,
                 arithmetic=ARITH_ACCURATE, adjoint=False, autotune=False):
        if isinstance(scenes, Scene):
            scenes = [scenes]
        self.scenes = list(scenes)
        arr = (SceneDesc * len(self.scenes))(*[s.desc for s in self.scenes])
        self._arr = arr
        opt = Options(precision, max_steps, 1 if use_graphs else 0, device, 1 if autotune else 0, arithmetic,
                      1 if adjoint else 0)
        h = C.c_void_p()
        _check(lib().ard_create(arr, len(self.scenes), C.byref(opt), C.byref(h)))
        self._h = h
        self.max_steps = max_steps
        self.precision = precision

    def close(self):
        if getattr(self, "_h", None):
            lib().ard_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _c(self, rc):
        _check(rc, self._h)

    def set_source_series(self, source, series, scene=0):
        s = np.ascontiguousarray(series, np.float32)
        self._c(lib().ard_set_source_series(self._h, scene, source, _fptr(s), s.size))

    def set_source_samples(self, t0, samples, source=-1, scene=-1):
        """Samples t0 .. t0+n-1 of one source's series (source, scene >= 0:
        `samples` is [n]) or of every source (-1, -1: [n_sources_total][n])."""
        s = np.ascontiguousarray(samples, np.float32)
        n = s.shape[-1] if s.ndim else 0
        self._c(lib().ard_set_source_samples(self._h, scene, source, t0, n, _fptr(s)))

    def set_initial_pressure(self, partition, pressure, scene=0):
        p = np.ascontiguousarray(pressure, np.float32)
        self._c(lib().ard_set_initial_pressure(self._h, scene, partition, _fptr(p)))

    def set_pml_scale(self, scale6, scene=0):
        s = np.ascontiguousarray(scale6, np.float32)
        self._c(lib().ard_set_pml_scale(self._h, scene, _fptr(s)))

    def reset(self):
        self._c(lib().ard_reset(self._h))

    def run(self, n, stream=None):
        self._c(lib().ard_step(self._h, n, stream))

    def Update(self):
        """One step; returns the step index before the increment (simulation.cpp:302)."""
        t = self.time_step
        self.run(1)
        return t

    STAGES = ("pml", "fwd_rows", "fwd_cols", "modal", "recorder", "inv_cols", "inv_rows", "iface")

    def profile(self, n, stream=None):
        """Mean device ms per step of each stage over n un-captured steps."""
        out = np.zeros(8, np.float32)
        self._c(lib().ard_profile_steps(self._h, n, stream, _fptr(out), 8))
        return dict(zip(self.STAGES, out.tolist()))

    def synchronize(self):
        self._c(lib().ard_synchronize(self._h))

    @property
    def layout(self):
        """The layout choices of the context (ard_describe)."""
        b = C.create_string_buffer(4096)
        self._c(lib().ard_describe(self._h, b, 4096))
        return b.value.decode()

    @property
    def kernels_per_step(self):
        v = C.c_int32()
        self._c(lib().ard_kernels_per_step(self._h, C.byref(v)))
        return v.value

    @property
    def time_step(self):
        v = C.c_int64()
        self._c(lib().ard_time_step(self._h, C.byref(v)))
        return v.value

    def recorders(self, scene=0, t0=0, nt=None, f64=False):
        """Recorder samples [nt][n_recorders]; scene=-1: every scene's recorders."""
        nt = self.time_step - t0 if nt is None else nt
        if scene == -1:
            nrec = sum(s.desc.n_recorders for s in self.scenes)
        elif 0 <= scene < len(self.scenes):
            nrec = self.scenes[scene].desc.n_recorders
        else:
            raise ArdError(6, f"bad scene index {scene}")
        if f64:
            out = np.zeros((nt, nrec), np.float64)
            self._c(lib().ard_read_recorders_f64(self._h, scene, out.ctypes.data_as(C.POINTER(C.c_double)), t0, nt))
        else:
            out = np.zeros((nt, nrec), np.float32)
            self._c(lib().ard_read_recorders(self._h, scene, _fptr(out), t0, nt))
        return out

    def adjoint(self, T, target, checkpoint_every=0, want_scale=True):
        """Gradients of J = 0.5 sum_{t<T} sum_r (rec[t][r] - target[t][r])^2 per scene
        (ard_adjoint).  `target`: [T][n_recorders] for one scene, or a list of
        such arrays, one per scene.  Runs the forward from step 0 itself.
        Returns dict(loss [n_scenes], grad_source [n_sources_total][T],
        grad_scale [n_scenes][6] or None)."""
        parts = target if isinstance(target, (list, tuple)) else [target]
        if len(parts) != len(self.scenes):
            raise ArdError(1, "one target array per scene")
        tg = np.concatenate([np.ascontiguousarray(t, np.float32).reshape(T, -1).ravel() for t in parts])
        nsrc = sum(s.desc.n_sources for s in self.scenes)
        gsrc = np.zeros((max(nsrc, 1), T), np.float32)
        gsc = np.zeros((len(self.scenes), 6), np.float32) if want_scale else None
        loss = np.zeros(len(self.scenes), np.float32)
        self._c(lib().ard_adjoint(self._h, T, _fptr(tg), checkpoint_every, _fptr(gsrc),
                                  _fptr(gsc) if want_scale else None, _fptr(loss)))
        return {"loss": loss, "grad_source": gsrc[:nsrc], "grad_scale": gsc}

    def initial_pressure_grad(self, partition, scene=0):
        """dJ/d(initial pressure) of an air partition after adjoint(), [z][y][x]."""
        if not (0 <= scene < len(self.scenes)) or not (0 <= partition < self.scenes[scene].desc.n_partitions):
            raise ArdError(6, f"bad scene/partition index {scene}/{partition}")
        q = self.scenes[scene].partitions[partition]
        out = np.zeros((q[7], q[6], q[5]), np.float32)
        self._c(lib().ard_read_initial_pressure_grad(self._h, scene, partition, _fptr(out)))
        return out

    def record_neighbourhoods(self, enable=True):
        """Record the 10x10x10 pressure cube around every recorder after every
        following step (Recorder::RecordField's out_ stream; ard_record_neighbourhoods)."""
        self._c(lib().ard_record_neighbourhoods(self._h, 1 if enable else 0))

    def neighbourhoods(self, scene=0, t0=0, nt=None):
        """Recorded cubes [nt][n_recorders][10][10][10] ([z][y][x] offsets -5 .. 4)."""
        nt = self.time_step - t0 if nt is None else nt
        nrec = (sum(s.desc.n_recorders for s in self.scenes) if scene == -1
                else self.scenes[scene].desc.n_recorders)
        out = np.zeros((nt, nrec, 10, 10, 10), np.float32)
        self._c(lib().ard_read_neighbourhoods(self._h, scene, _fptr(out), t0, nt))
        return out

    def slice_size(self, look_from=0, scene=0):
        w, h = C.c_int32(), C.c_int32()
        self._c(lib().ard_slice_size(self._h, scene, look_from, C.byref(w), C.byref(h)))
        return w.value, h.value

    def render_slice(self, look_from=0, coord=None, v_coef=10.0, scene=0, pixels=None, pressure=None):
        """Colour map of a pressure slice (Simulation::Update's visualization,
        ard_render_slice) into device buffers: `pixels` an int32 CUDA tensor of
        [height][width] RGBA8888 words (allocated zeroed when None), `pressure`
        an optional float32 CUDA tensor of the same shape.  coord defaults to
        the first source's z (xy) or x (yz), as the reference takes it."""
        import torch
        w, h = self.slice_size(look_from, scene)
        if coord is None:
            src = self.scenes[scene].sources[0]
            coord = src[2] if look_from == 0 else src[0]
        dev = torch.device("cuda", torch.cuda.current_device())
        if pixels is None:
            pixels = torch.zeros((h, w), dtype=torch.int32, device=dev)
        self._c(lib().ard_render_slice(self._h, scene, look_from, int(coord), float(v_coef),
                                       C.c_void_p(pixels.data_ptr()),
                                       C.c_void_p(pressure.data_ptr()) if pressure is not None else None))
        return pixels

    def impulse_response(self, nt=None, recorder=0, source=0, scene=0, truncate=0, sample_rate=0.0, fcut=3000.0,
                         fir_order=1024):
        """Room impulse response and T60 of matlab/auralization.m and t60.m on
        the device (ard_impulse_response).  Returns (rir [nt] float64,
        dict(t60_ms, slope, stop, overrun))."""
        nt = self.time_step if nt is None else nt
        rir = np.zeros(nt, np.float64)
        t60 = np.zeros(4, np.float64)
        dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
        self._c(lib().ard_impulse_response(self._h, scene, recorder, source, nt, truncate, sample_rate, fcut,
                                           fir_order, dp(rir), dp(t60)))
        return rir, dict(t60_ms=float(t60[0]), slope=float(t60[1]), stop=int(t60[2]), overrun=bool(t60[3]))

    def write_outputs(self, directory, scene=0, nt=None):
        """response_<r>.txt and source_<s>.txt in the reference's format, and
        out_<r>.txt when the neighbourhoods are recorded (ard_write_outputs)."""
        nt = self.time_step if nt is None else nt
        self._c(lib().ard_write_outputs(self._h, scene, os.fsencode(directory), nt))

    def field(self, partition, scene=0):
        if not (0 <= scene < len(self.scenes)) or not (0 <= partition < self.scenes[scene].desc.n_partitions):
            raise ArdError(6, f"bad scene/partition index {scene}/{partition}")
        q = self.scenes[scene].partitions[partition]
        out = np.zeros((q[7], q[6], q[5]), np.float32)
        self._c(lib().ard_read_field(self._h, scene, partition, _fptr(out)))
        return out
