"""Benchmark of the GB300 ARD time step.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--config c1] [--impl ours|reference]

One benchmark step is one full simulation of the workload: reset, then
`sim_steps` time steps (c1: the reference's scene-3 L-shaped room at
h = 0.025 m, 8000 steps).  Metric: air-cell steps per second (Gcell-steps/s),
the cells of the air (DCT) partitions advanced one time step; PML cells are
extra work, not counted.

  value   device-resident: K simulations timed with CUDA events on the
          launching stream, L2 flushed (256 MiB write) before each
  e2e     the same through the public API with host buffers: per simulation
          upload the source series from pinned memory, reset, step, read the
          recorder history back
  roofline  the modal kernel (the dominant stage): algorithmic bytes per
          launch (28 B per air cell, the reference's per-cell reads and
          writes of one air-partition update) over its CUDA-event time
          (ard_profile_steps: the step's stages launched directly on one
          stream, events around each stage, averaged over min(sim_steps,
          200) steps in this process), against the measured HBM copy bandwidth; traffic = the
          kernel's DRAM bytes per launch from the ncu summary in profiles/
  cpu_baseline  the oracle (C restatement of the reference's CPU solver,
          FP32, OpenMP over partitions) on a bounded sample of the same scene
  accuracy  FP32 recorders against the FP64 GPU path (same kernels in
          double) on a bounded sample of the workload
  adjoint the forward + adjoint of the recorder misfit on the same workload
          (gradients w.r.t. source series, initial pressure and the six PML
          face scales; target from a seeded perturbed source, face scales
          U(0.5, 1.5); --checkpoint-every K, 0 = the library's choice: the
          whole PML history when it fits): wall time against the forward
          alone, and Gcell-steps/s of forward + adjoint
  --plain runs every scene in its own context one after another (the
          per-scene path) instead of one batched context

Multi-GPU (torchrun): scenes are independent, so ranks shard the scene list
(c2) or run replicas (single-scene configs); no collective touches the data
path.  --impl reference times the reference's CPU algorithm (the oracle port;
the reference sources are not on the GPU machine) on rank 0.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "ard-simulator_gb300"))

METRIC = "Gcell-steps/s fwd & fwd+adjoint on 1 GB300 at ≤1e-4 rel recorder err vs FP64"
UNIT = "Gcell-steps/s"
BYTES_PER_AIR_CELL = 28      # read f, M, M_prev, cos, psi; write M_next, p (4 B each)
MODAL_STAGE = "modal"


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def workload(name, sim_steps=None, rank=0, world=1):
    from ard_gb300 import configs as K
    from ard_gb300 import shard
    cfg = K.config(name, steps=sim_steps)
    scenes = cfg["scenes"]
    # independent scenes: balanced shards by air cells (a single scene is replicated)
    costs = [sum(b[3] * b[4] * b[5] for b in sc["air"]) for sc in scenes]
    cfg["scenes"] = [scenes[i] for i in shard.local_scenes(costs, rank, world)]
    return cfg


def describe(cfg, n_air, n_pml):
    return (f"{cfg['name']}: {len(cfg['scenes'])} scene(s), {n_air} air cells, {n_pml} PML cells, "
            f"h={cfg['h']} m, {cfg['pml']}-cell PML, {cfg['steps']} steps per simulation")


class ClockSampler:
    """nvidia-smi clocks and throttle reasons while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits", "-lms", "200",
                 "-i", str(self.device)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.thread.join(timeout=2)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_baseline(cfg, sample_steps, target_s=0.0):
    """The oracle (C restatement of the reference CPU solver, FP32) on the
    first scene of the workload, all host threads: at least `sample_steps`
    steps, continued (in chunks of about a second) until `target_s` seconds
    of stepping, within the scene's series length."""
    from oracle import oracle as O
    sc = cfg["scenes"][0]
    params = dict(dh=float(np.float32(cfg["h"])), dt=cfg["dt"], c0=float(np.float32(cfg["c0"])),
                  pml_layers=cfg["pml"])
    flat = O.make_flat_scene(sc["air"], sc["sources"], sc["recorders"], params)
    sim = O.OracleSim(flat, "f32")
    for i, s in enumerate(sc["series"]):
        sim.set_source_series(i, s)
    sim.step(1)  # first-touch allocation outside the timing
    limit = max(sample_steps, int(cfg["steps"]) - 1)
    t0 = time.perf_counter()
    sim.step(sample_steps)
    el = time.perf_counter() - t0
    while el < target_s and sample_steps < limit:
        chunk = max(1, min(limit - sample_steps, int(sample_steps / max(el, 1e-6))))
        sim.step(chunk)
        sample_steps += chunk
        el = time.perf_counter() - t0
    n_air = sum(b[3] * b[4] * b[5] for b in sc["air"])
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    return dict(value=n_air * sample_steps / el / 1e9, unit=UNIT, cores=cores, kind="port",
                sample=f"{sample_steps} steps of scene 0 of {cfg['name']} ({n_air} air cells), "
                       f"oracle/ard_oracle.c FP32, OpenMP over partitions, {el:.2f} s")


def run_reference_arm(args, rank):
    if rank != 0:
        return 0
    os.environ.setdefault("OMP_NUM_THREADS", str(os.cpu_count() or 1))
    cfg = workload(args.config, args.sim_steps)
    sample = args.ref_sample
    per = []
    for i in range(args.warmup + args.steps):
        cb = cpu_baseline(cfg, sample)
        if i >= args.warmup:
            per.append(cb["value"])
    value = statistics.median(per)
    n_air = sum(b[3] * b[4] * b[5] for sc in cfg["scenes"][:1] for b in sc["air"])
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": n_air * sample / value / 1e6, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "impl": "reference",
            "config": {"workload": describe(cfg, n_air, 0), "sample_steps": sample},
            "cpu_baseline": dict(cb, value=value),
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def accuracy_measurement(A, cfg, scenes, args, device):
    """Recorder error of the FP32 product path against the FP64 GPU oracle
    (the same kernels in double) on a bounded sample: the first 16 scenes,
    min(steps, 2000) steps for multi-scene or c4-size workloads, the whole
    run otherwise.  Relative L2 per recorder; the max is reported."""
    S = cfg["steps"]
    n_air = sum(s.air_cells for s in scenes)
    big = len(scenes) > 1 or n_air > 5e7
    T = min(S, 2000) if big else S
    sub = scenes[:16]
    subcfg = cfg["scenes"][:16]
    out = []
    for prec in (A.PREC_F32, A.PREC_F64):
        sim = A.Simulation(sub, precision=prec, max_steps=T, device=device)
        k = 0
        for i, sc in enumerate(subcfg):
            for j, srs in enumerate(sc["series"]):
                sim.set_source_series(j, srs[:T], scene=i)
        sim.run(T)
        out.append(sim.recorders(scene=-1, f64=True))
        sim.close()
    a, b = out
    # recorders the wave has reached: RMS above 1e-3 of the loudest recorder's (the others
    # hold only the rounding noise of the global modal transforms, where a relative error means nothing)
    rms = np.sqrt(np.mean(b ** 2, axis=0))
    live = [r for r in range(b.shape[1]) if rms[r] > 1e-3 * rms.max()]
    errs = [float(np.linalg.norm(a[:, r] - b[:, r]) / np.linalg.norm(b[:, r])) for r in live]
    return {"rel_l2_vs_fp64_max": max(errs) if errs else None, "recorders": len(live),
            "recorders_total": int(b.shape[1]),
            "rel_l2_vs_fp64_all": float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)),
            "sample": f"{len(sub)} scene(s), {T} steps, FP32 accurate arithmetic vs FP64 GPU; max over recorders "
                      f"whose RMS is above 1e-3 of the loudest"}


def adjoint_measurement(A, cfg, scenes, args, device):
    """Forward + adjoint of the recorder misfit (gradients w.r.t. the source
    series, the initial pressure and the six PML face scales) against the
    forward alone, on the bench workload.  Target: recorders of a run whose
    sources carry seeded band-limited noise on top of the series; face scales
    U(0.5, 1.5), seeded."""
    import torch
    S = args.adjoint_steps or cfg["steps"]
    rng = np.random.default_rng(7)
    sim = A.Simulation(scenes, max_steps=S, device=device, adjoint=True)
    n_src = sum(len(sc["sources"]) for sc in cfg["scenes"])
    series = np.zeros((n_src, S), np.float32)
    k = 0
    for sc in cfg["scenes"]:
        for s in sc["series"]:
            series[k] = s[:S]
            k += 1
    amp = float(np.abs(series).max()) or 1.0
    noise = rng.standard_normal((n_src, S))
    spec = np.fft.rfft(noise, axis=1)
    f = np.fft.rfftfreq(S, d=cfg["dt"])
    spec[:, f > 2000.0] = 0                      # 2 kHz band limit
    pert = (0.1 * amp * np.fft.irfft(spec, n=S, axis=1) / (np.abs(np.fft.irfft(spec, n=S, axis=1)).max() + 1e-30))
    pert[:, 1024:] = 0                           # 1024 samples of noise, then zeros
    scales = rng.uniform(0.5, 1.5, size=(len(scenes), 6)).astype(np.float32)

    def load(series_):
        sim.reset()
        sim._c(A.lib().ard_set_source_series(sim._h, -1, -1, A._fptr(np.ascontiguousarray(series_, np.float32)), S))
        for i in range(len(scenes)):
            sim.set_pml_scale(scales[i], scene=i)

    load(series + pert.astype(np.float32))
    sim.run(S)
    target = sim.recorders(scene=-1)
    tparts, r0 = [], 0
    for sc in cfg["scenes"]:
        n = len(sc["recorders"])
        tparts.append(target[:, r0:r0 + n])
        r0 += n
    load(series)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    sim.run(S)
    sim.synchronize()
    fwd_s = time.perf_counter() - t0
    load(series)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    g = sim.adjoint(S, tparts, checkpoint_every=args.checkpoint_every, want_scale=True)
    adj_s = time.perf_counter() - t0
    n_air = sum(s.air_cells for s in scenes)
    out = {"workload": f"{cfg['name']} geometry, {S} steps, checkpoint every {args.checkpoint_every}",
           "path": sim.layout.split("last adjoint: ")[-1],
           "fwd_s": fwd_s, "fwd_adj_s": adj_s, "ratio": adj_s / fwd_s,
           "value": n_air * S / adj_s / 1e9, "unit": UNIT,
           "loss": float(np.sum(g["loss"])),
           "grad_scale_scene0": [float(v) for v in g["grad_scale"][0]]}
    sim.close()
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--config", default="c1")
    ap.add_argument("--sim-steps", type=int, default=None, help="time steps per simulation (default: config)")
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-sample", type=int, default=2, help="minimum time steps of the CPU baseline sample")
    ap.add_argument("--cpu-seconds", type=float, default=10.0,
                    help="the CPU baseline steps on until this many seconds (within the series length)")
    ap.add_argument("--ref-sample", type=int, default=6, help="time steps per reference-arm step")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--no-accuracy", action="store_true")
    ap.add_argument("--adjoint-steps", type=int, default=None, help="steps of the adjoint measurement (default: sim steps)")
    ap.add_argument("--checkpoint-every", type=int, default=0,
                    help="adjoint checkpoint interval (0: keep the whole PML history when it fits, else automatic)")
    ap.add_argument("--plain", action="store_true", help="one context per scene, run one after another")
    ap.add_argument("--autotune", action="store_true", help="let ard_create time candidate layouts and keep the fastest")
    ap.add_argument("--adjoint-only", action="store_true",
                    help="only the forward + adjoint measurement (one line with the adjoint object)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3) if args.impl == "ours" else args.warmup

    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    local = int(os.environ.get("LOCAL_RANK", 0))
    if args.impl == "reference":
        return run_reference_arm(args, rank)

    import torch
    import ard_gb300 as A

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    cfg = workload(args.config, args.sim_steps, rank, world)
    S = cfg["steps"]
    h32 = float(np.float32(cfg["h"]))
    scenes = [A.build_scene(sc["air"], sc["sources"], sc["recorders"], h32, cfg["dt"], cfg["c0"], cfg["pml"])
              for sc in cfg["scenes"]]
    if args.adjoint_only:
        adj = adjoint_measurement(A, cfg, scenes, args, local)
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": adj["value"], "unit": UNIT, "n_gpus": world,
                              "steps": 1, "warmup": 0, "ms_per_step": adj["fwd_adj_s"] * 1e3,
                              "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                              "data": "synthetic", "config": {"workload": adj["workload"]}, "adjoint": adj}),
                  flush=True)
        return 0
    n_air = sum(s.air_cells for s in scenes)
    n_pml = sum(s.pml_cells for s in scenes)
    n_src = sum(len(sc["sources"]) for sc in cfg["scenes"])
    n_rec = sum(len(sc["recorders"]) for sc in cfg["scenes"])
    sims = [A.Simulation([sc], max_steps=S, device=local, autotune=args.autotune) for sc in scenes] if args.plain else None
    sim = sims[0] if args.plain else A.Simulation(scenes, max_steps=S, device=local, autotune=args.autotune)
    series = np.zeros((n_src, S), np.float32)
    k = 0
    for sc in cfg["scenes"]:
        for s in sc["series"]:
            series[k] = s[:S]
            k += 1
    pinned_series = torch.from_numpy(series).pin_memory()
    pinned_rec = torch.empty((S, n_rec), dtype=torch.float32).pin_memory()
    import ctypes as C
    fptr = lambda t: C.cast(t.data_ptr(), C.POINTER(C.c_float))

    if args.plain:
        # per-scene contexts: each takes its own rows of the series / recorder buffers
        src_off = np.cumsum([0] + [len(sc["sources"]) for sc in cfg["scenes"]])
        rec_off = np.cumsum([0] + [len(sc["recorders"]) for sc in cfg["scenes"]])
        rec_rows = [torch.empty((S, int(rec_off[i + 1] - rec_off[i])), dtype=torch.float32).pin_memory()
                    for i in range(len(sims))]

    def upload():
        if not args.plain:
            sim._c(A.lib().ard_set_source_series(sim._h, -1, -1, fptr(pinned_series), S))
            return
        for i, sm in enumerate(sims):
            if src_off[i + 1] > src_off[i]:
                sm._c(A.lib().ard_set_source_series(sm._h, -1, -1, fptr(pinned_series[int(src_off[i]):]), S))

    def readback():
        if not args.plain:
            sim._c(A.lib().ard_read_recorders(sim._h, -1, fptr(pinned_rec), 0, S))
            return
        for i, sm in enumerate(sims):
            if rec_off[i + 1] > rec_off[i]:
                sm._c(A.lib().ard_read_recorders(sm._h, -1, fptr(rec_rows[i]), 0, S))

    def reset_all():
        for sm in (sims if args.plain else [sim]):
            sm.reset()

    def run_all(n, stream=None):
        for sm in (sims if args.plain else [sim]):
            sm.run(n, stream=stream)

    upload()
    stream = torch.cuda.Stream()
    handle = stream.cuda_stream
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")   # 256 MiB > 129 MB L2

    def simulate():
        reset_all()
        with torch.cuda.stream(stream):
            flush.fill_(1.0)
        run_all(S, stream=handle)

    for _ in range(args.warmup):
        simulate()
    torch.cuda.synchronize()

    # ---- device-resident timed region ----
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    total_ms = 0.0
    for _ in range(args.steps):
        reset_all()
        with torch.cuda.stream(stream):
            flush.fill_(1.0)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
        run_all(S, stream=handle)
        with torch.cuda.stream(stream):
            e1.record(stream)
        e1.synchronize()
        total_ms += e0.elapsed_time(e1)
    torch.cuda.synchronize()
    clk = clocks.stop()
    if dist:
        t = torch.tensor([total_ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
        tot = torch.tensor([float(n_air)], device="cuda", dtype=torch.float64)
        dist.all_reduce(tot)
        n_air_all = float(tot.item())
    else:
        n_air_all = float(n_air)
    value = n_air_all * S * args.steps / (total_ms / 1e3) / 1e9
    ms_per_step = total_ms / args.steps

    # ---- end to end through the public API (host buffers, pinned) ----
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        upload()
        reset_all()
        run_all(S)
        readback()
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    if dist:
        t = torch.tensor([e2e_s], device="cuda", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t.item())
    e2e = {"value": n_air_all * S * args.steps / e2e_s / 1e9, "unit": UNIT,
           "h2d_bytes_per_step": int(series.nbytes), "d2h_bytes_per_step": int(S * n_rec * 8)}

    # ---- per-stage device times (un-captured steps, CUDA events per kernel) ----
    sim.reset()
    with torch.cuda.stream(stream):
        flush.fill_(1.0)
    prof_steps = min(S, 200)
    stages = sim.profile(prof_steps, stream=handle)
    peak, peak_kind = peaks()
    modal_ms = stages[MODAL_STAGE]
    # the profiled context: the batch, or (plain) the first scene's own context
    alg_bytes = BYTES_PER_AIR_CELL * (scenes[0].air_cells if args.plain else n_air)
    achieved = alg_bytes / (modal_ms / 1e3) / 1e9 if modal_ms > 0 else 0.0
    traffic = None
    tpath = os.path.join(ROOT, "profiles", f"traffic_{args.config}.txt")
    if os.path.exists(tpath):
        with open(tpath) as f:
            for ln in f:
                if ln.startswith("modal_kernel_dram_bytes_per_launch:"):
                    traffic = int(ln.split(":")[1])
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": traffic, "peak_source": peak_kind,
                "kernel": "modal_kernel<float>", "algorithmic_bytes_per_launch": alg_bytes,
                "launch_ms": modal_ms}
    # whole step: the reference's per-step algorithmic bytes over the device time of one step
    n_face = sum(s.face_cells for s in scenes)
    step_bytes = 28 * n_air + 44 * n_pml + 48 * n_face
    step_roofline = {"algorithmic_bytes_per_step": step_bytes, "ms_per_step": ms_per_step / S,
                     "achieved": step_bytes / (ms_per_step / S / 1e3) / 1e9, "unit": "GB/s",
                     "frac": step_bytes / (ms_per_step / S / 1e3) / 1e9 / peak}
    kps = sum(sm.kernels_per_step for sm in (sims if args.plain else [sim]))
    launches = int(args.steps * (S * kps + (S // 32 + S % 32) * (len(sims) if args.plain else 1)))

    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": describe(cfg, n_air, n_pml), "sim_steps_per_step": S,
                       "scenes_per_rank": len(scenes), "parallelism": "replicas" if len(cfg["scenes"]) == 1 else "scene shards",
                       "l2": "flushed (256 MiB write) before every timed simulation; the scene's working set may fit in L2 within a simulation"},
            "roofline": roofline,
            "step_roofline": step_roofline,
            "stage_ms_per_step": stages,
            "e2e": e2e,
            "gpu_launches": launches,
            "kernels_per_step": kps,
            "clocks": clk}
    line["config"]["layout"] = sim.layout
    if not args.no_accuracy and not args.plain:
        line["accuracy"] = accuracy_measurement(A, cfg, scenes, args, local)
    if args.plain:
        line["config"]["parallelism"] = "plain: one context per scene, run one after another"
    if not args.no_adjoint and not args.plain:
        line["adjoint"] = adjoint_measurement(A, cfg, scenes, args, local)
    if rank == 0 and not args.no_cpu_baseline:
        os.environ.setdefault("OMP_NUM_THREADS", str(os.cpu_count() or 1))
        line["cpu_baseline"] = cpu_baseline(cfg, args.cpu_sample, args.cpu_seconds)
    if rank == 0:
        print(json.dumps(line), flush=True)
    sim.close()
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
