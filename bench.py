"""Benchmark of the GB300 ARD time step.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--config c4] [--impl ours|reference]

Workload (default c4): the 40 x 25 m hall, 12 m deep, 24 air partitions at
h = 0.04 m (187.5 M air cells, 10-cell PML, 16 recorders), 20000 time steps.
One benchmark step is `chunk` consecutive time steps of one simulation (1000
for c4, so `--steps 20` covers the configured 20000 steps once; the state
carries from one benchmark step to the next, and the simulation restarts
from rest when it reaches its configured length).  Workloads of fewer than
10000 steps take a whole simulation per benchmark step.  Metric: air-cell
steps per second (Gcell-steps/s), the cells of the air (DCT) partitions
advanced one time step; PML cells are extra work, not counted.

  value   device time of the benchmark steps, CUDA events on the launching
          stream around each step's ard_step call (inputs resident in HBM;
          the c4 state, ~5 GB, is far larger than L2; L2 is also flushed
          with a 256 MiB write before every benchmark step)
  e2e     the same steps end to end through the C ABI, host wall clock:
          per benchmark step the upload of that step's source samples from
          pinned host memory (ard_set_source_samples), the steps, and the
          read-back of that step's recorder samples (ard_read_recorders)
  roofline  the modal kernel (the dominant HBM-bound stage): algorithmic
          bytes per launch (28 B per air cell, the reference's per-cell
          reads and writes of one air-partition update) over its CUDA-event
          time (ard_profile_steps: the stages of min(steps, 200) un-captured
          steps launched on one stream with events around each), against
          the measured HBM copy bandwidth; traffic = the kernel's DRAM bytes
          per launch from the ncu summary in profiles/
  stage_roofline  every stage against its bound: PML 44 B per PML cell,
          interfaces 48 B per face cell, modal 28 B per air cell (HBM), the
          face transforms as useful FLOP/s (and, on the tensor-core path, the
          split-TF32 product rate against the dense TF32 rate) and as bytes
          moved against HBM
  reference_arithmetic  the same workload in the reference's FP32
          arithmetic (the mode that reproduces the reference CPU solver's
          rounding), timed the same way on a shorter run
  accuracy  recorders of the FP32 runs against the FP64 GPU path (the same
          kernels in double)
  adjoint the forward + adjoint of the recorder misfit at the workload's
          length (gradients w.r.t. source series, initial pressure and the
          six PML face scales; the adjoint's forward run injects the series
          plus seeded band-limited noise (1024 samples, 2 kHz), the target
          is the recorder signal of the timed forward run; face scales
          U(0.5, 1.5), seeded): wall time of the ard_adjoint call against the
          device time of the forward steps
  batched_vs_plain  the first 16 scenes of the batched workload (c2) for 320
          steps in one context against one context per scene run one after
          another, host wall clock
  cpu_baseline  the oracle (C restatement of the reference's CPU solver,
          FP32, OpenMP over partitions) on a bounded sample of the same scene
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
BYTES_PER_PML_CELL = 44      # read p, p_prev, phi x3, f; write p_next, phi x3, clear f
BYTES_PER_FACE_CELL = 48     # 6 reads + 6 writes per interface face cell
MODAL_STAGE = "modal"
FP32_FMA_TFLOPS = 152 * 128 * 2 * 2.07e9 / 1e12   # CUDA-core FP32 peak at the 2070 MHz maximum SM clock


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


def default_chunk(steps):
    """Time steps per benchmark step: 1000 for long runs (c4), else a whole simulation."""
    return 1000 if steps >= 10000 else steps


def describe(cfg, n_air, n_pml):
    return (f"{cfg['name']}: {len(cfg['scenes'])} scene(s), {n_air} air cells, {n_pml} PML cells, "
            f"h={cfg['h']} m, {cfg['pml']}-cell PML, {cfg['steps']} steps per simulation")


def face_flops(scenes):
    """Useful FLOPs of one step's face transforms: per air partition and axis,
    forward and inverse each six 2D transforms (three layer pairs, even and
    odd parts) of a V x U face, V U (U + V) multiply-adds each."""
    total = 0
    for sc in scenes:
        for p in sc.partitions:
            if p[0] != 0:
                continue
            w, h, d = p[5], p[6], p[7]
            macs = d * h * (d + h) + d * w * (d + w) + h * w * (h + w)
            total += 2 * 2 * 6 * macs
    return total


def face_bytes(scenes):
    """Algorithmic bytes of one step's four face-transform passes (FP32): each
    pass reads its input layers and writes its output layers once, the first
    pass of each direction reading the two layers of every pair (forward:
    the force faces, inverse: the contraction sums): 2 + 1 + 1 (forward) and
    2 + 1 + 1 (inverse) reads plus 4 writes of the 18 face layers."""
    total = 0
    for sc in scenes:
        for p in sc.partitions:
            if p[0] != 0:
                continue
            w, h, d = p[5], p[6], p[7]
            fe = 6 * (d * h + d * w + h * w)
            total += 4 * 10 * fe
    return total


def tf32_peak_tflops():
    """Dense TF32 tensor rate: half the measured dense bf16 rate (the
    tensor cores' TF32 rate is half their bf16 rate)."""
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            return float(json.load(f)["bf16_tflops"]) / 2, "measured bf16 / 2"
    return 1900.0 / 2, "fallback bf16 / 2"


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
        sm, mx, pw, reasons = [], [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
                pw.append(float(parts[3]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm), "power_w_max": max(pw) if pw else None}


def oracle_scene(cfg):
    """The oracle (FP32) on the first scene of the workload, with its series
    set; returns (sim, air cells, PML cells, setup seconds)."""
    from oracle import oracle as O
    sc = cfg["scenes"][0]
    params = dict(dh=float(np.float32(cfg["h"])), dt=cfg["dt"], c0=float(np.float32(cfg["c0"])),
                  pml_layers=cfg["pml"])
    t0 = time.perf_counter()
    flat = O.make_flat_scene(sc["air"], sc["sources"], sc["recorders"], params)
    sim = O.OracleSim(flat, "f32")
    for i, s in enumerate(sc["series"]):
        sim.set_source_series(i, s)
    n_air = sum(p[5] * p[6] * p[7] for p in flat["partitions"] if p[0] == 0)
    n_pml = sum(p[5] * p[6] * p[7] for p in flat["partitions"] if p[0] == 1)
    return sim, n_air, n_pml, time.perf_counter() - t0


def cpu_threads():
    return int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))


def cpu_baseline(cfg, sample_steps, target_s=0.0):
    """The oracle (C restatement of the reference CPU solver, FP32) on the
    first scene of the workload, all host threads: at least `sample_steps`
    steps, continued (in chunks of about a second) until `target_s` seconds
    of stepping, within the scene's series length."""
    sim, n_air, n_pml, _ = oracle_scene(cfg)
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
    sim.close()
    return dict(value=n_air * sample_steps / el / 1e9, unit=UNIT, cores=cpu_threads(), kind="port",
                sample=f"{sample_steps} steps of scene 0 of {cfg['name']} ({n_air} air cells, {n_pml} PML cells), "
                       f"oracle/ard_oracle.c FP32, OpenMP over partitions, {el:.2f} s")


def run_reference_arm(args, rank):
    """The reference's CPU algorithm (the oracle port, all host threads) on
    the same workload: the scene is built once, then every benchmark step
    advances it by `--ref-sample` time steps (a bounded sample of the
    benchmark step's work; the metric is per air-cell step)."""
    if rank != 0:
        return 0
    os.environ.setdefault("OMP_NUM_THREADS", str(os.cpu_count() or 1))
    cfg = workload(args.config, args.sim_steps)
    sample = args.ref_sample or (1 if cfg["steps"] >= 10000 else 6)
    sim, n_air, n_pml, setup_s = oracle_scene(cfg)
    sim.step(1)  # first-touch allocation outside the timing
    per = []
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        sim.step(sample)
        el = time.perf_counter() - t0
        if i >= args.warmup:
            per.append(el)
    sim.close()
    total = sum(per)
    value = n_air * sample * len(per) / total / 1e9
    cb = dict(value=value, unit=UNIT, cores=cpu_threads(), kind="port",
              sample=f"{sample} time step(s) of scene 0 of {cfg['name']} per benchmark step ({n_air} air cells, "
                     f"{n_pml} PML cells), oracle/ard_oracle.c FP32, OpenMP over partitions, {total:.2f} s "
                     f"over {len(per)} benchmark steps (setup {setup_s:.1f} s, untimed)")
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total / len(per) * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "impl": "reference",
            "config": {"workload": describe(cfg, n_air, n_pml), "sample_steps_per_step": sample},
            "cpu_baseline": cb,
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def rel_errors(a, b):
    """Relative L2 error per recorder of a against b ([T][R]), over the
    recorders the wave has reached (RMS above 1e-3 of the loudest recorder's;
    the others hold only the rounding noise of the global modal transforms,
    where a relative error means nothing)."""
    rms = np.sqrt(np.mean(b ** 2, axis=0))
    live = [r for r in range(b.shape[1]) if rms[r] > 1e-3 * rms.max()]
    errs = [float(np.linalg.norm(a[:, r] - b[:, r]) / np.linalg.norm(b[:, r])) for r in live]
    return (max(errs) if errs else None), live


def load_series(sim, cfg, T, scenes_slice=None):
    for i, sc in enumerate(cfg["scenes"] if scenes_slice is None else cfg["scenes"][scenes_slice]):
        for j, srs in enumerate(sc["series"]):
            sim.set_source_series(j, srs[:T], scene=i)


def run_recorders(A, cfg, scenes, T, device, **kw):
    sim = A.Simulation(scenes, max_steps=T, device=device, **kw)
    load_series(sim, cfg, T)
    sim.run(T)
    out = sim.recorders(scene=-1, f64=True)
    sim.close()
    return out


def accuracy_measurement(A, cfg, scenes, device, rec32=None, rec_ref=None):
    """Recorder error of the FP32 product path (accurate arithmetic; and the
    reference arithmetic when `rec_ref` is given) against the FP64 GPU
    oracle (the same kernels in double) on a bounded sample: the first 16
    scenes, min(steps, 2000) steps for multi-scene or c4-size workloads, the
    whole run otherwise.  `rec32` / `rec_ref`: FP32 recorders of the same
    steps already recorded by the benchmark (else run here)."""
    S = cfg["steps"]
    n_air = sum(s.air_cells for s in scenes)
    big = len(scenes) > 1 or n_air > 5e7
    T = min(S, 2000) if big else S
    sub = scenes[:16]
    subcfg = dict(cfg, scenes=cfg["scenes"][:16])
    if len(scenes) > 16 or rec32 is None or rec32.shape[0] < T:
        rec32 = run_recorders(A, subcfg, sub, T, device, precision=A.PREC_F32)
        rec_ref = None
    else:
        rec32 = rec32[:T]
    ref64 = run_recorders(A, subcfg, sub, T, device, precision=A.PREC_F64)
    emax, live = rel_errors(rec32, ref64)
    out = {"rel_l2_vs_fp64_max": emax, "recorders": len(live), "recorders_total": int(ref64.shape[1]),
           "rel_l2_vs_fp64_all": float(np.linalg.norm(rec32 - ref64) / max(np.linalg.norm(ref64), 1e-300)),
           "sample": f"{len(sub)} scene(s), {T} steps, FP32 accurate arithmetic vs FP64 GPU; max over recorders "
                     f"whose RMS is above 1e-3 of the loudest"}
    if rec_ref is not None and rec_ref.shape[0] >= T:
        out["reference_arithmetic_rel_l2_vs_fp64_max"] = rel_errors(rec_ref[:T], ref64)[0]
    return out


def band_limited_noise(rng, n_src, S, dt, amp):
    noise = rng.standard_normal((n_src, S))
    spec = np.fft.rfft(noise, axis=1)
    f = np.fft.rfftfreq(S, d=dt)
    spec[:, f > 2000.0] = 0                      # 2 kHz band limit
    x = np.fft.irfft(spec, n=S, axis=1)
    pert = 0.1 * amp * x / (np.abs(x).max() + 1e-30)
    pert[:, 1024:] = 0                           # 1024 samples of noise, then zeros
    return pert.astype(np.float32)


def adjoint_measurement(A, cfg, scenes, args, device, series, target, fwd_s_per_step):
    """Forward + adjoint of the recorder misfit (gradients w.r.t. the source
    series, the initial pressure and the six PML face scales) on the bench
    workload, `S` steps.  The adjoint's forward injects the series plus
    seeded band-limited noise; the target is the recorder signal of the
    timed forward run (`target`, [S][n_rec]); face scales U(0.5, 1.5),
    seeded.  The ratio is the ard_adjoint call's wall time over the device
    time of S forward steps measured by the benchmark."""
    S = target.shape[0]
    rng = np.random.default_rng(7)
    n_src = series.shape[0]
    amp = float(np.abs(series).max()) or 1.0
    pert = band_limited_noise(rng, n_src, S, cfg["dt"], amp)
    scales = rng.uniform(0.5, 1.5, size=(len(scenes), 6)).astype(np.float32)
    sim = A.Simulation(scenes, max_steps=S, device=device, adjoint=True)
    sim.set_source_samples(0, np.ascontiguousarray(series[:, :S] + pert))
    for i in range(len(scenes)):
        sim.set_pml_scale(scales[i], scene=i)
    tparts, r0 = [], 0
    for sc in cfg["scenes"]:
        n = len(sc["recorders"])
        tparts.append(np.ascontiguousarray(target[:, r0:r0 + n]))
        r0 += n
    sim.synchronize()
    t0 = time.perf_counter()
    g = sim.adjoint(S, tparts, checkpoint_every=args.checkpoint_every, want_scale=True)
    adj_s = time.perf_counter() - t0
    fwd_s = fwd_s_per_step * S
    n_air = sum(s.air_cells for s in scenes)
    out = {"workload": f"{cfg['name']} geometry, {S} steps (the whole simulation), checkpoint every "
                       f"{args.checkpoint_every or 'auto'}",
           "path": sim.layout.split("last adjoint: ")[-1],
           "fwd_s": fwd_s, "fwd_s_source": "device time of the benchmark's forward steps, per step x S",
           "fwd_adj_s": adj_s, "ratio": adj_s / fwd_s,
           "value": n_air * S / adj_s / 1e9, "unit": UNIT,
           "loss": float(np.sum(g["loss"])),
           "grad_scale_scene0": [float(v) for v in g["grad_scale"][0]]}
    sim.close()
    return out


def batching_measurement(A, device, n_scenes=16, T=320):
    """Batched against plain on the batched workload's scenes: the first
    `n_scenes` c2 scenes for T steps, in one context (one launch per stage
    over all scenes, the production path) and in one context per scene run
    one after another (the per-scene path), each after 64 warm-up steps and
    a reset; host wall clock around the runs and a synchronize after each."""
    cfg = workload("c2", T)
    cfg = dict(cfg, scenes=cfg["scenes"][:n_scenes])
    h32 = float(np.float32(cfg["h"]))
    scenes = [A.build_scene(sc["air"], sc["sources"], sc["recorders"], h32, cfg["dt"], cfg["c0"], cfg["pml"])
              for sc in cfg["scenes"]]
    n_air = sum(s.air_cells for s in scenes)

    def timed(groups):
        sims = []
        for g in groups:
            sim = A.Simulation([scenes[i] for i in g], max_steps=T, device=device)
            load_series(sim, dict(cfg, scenes=[cfg["scenes"][i] for i in g]), T)
            sim.run(64)
            sim.synchronize()
            sim.reset()
            sims.append(sim)
        t0 = time.perf_counter()
        for sim in sims:
            sim.run(T)
            sim.synchronize()
        dt = time.perf_counter() - t0
        for sim in sims:
            sim.close()
        return n_air * T / dt / 1e9

    batched = timed([list(range(len(scenes)))])
    plain = timed([[i] for i in range(len(scenes))])
    return {"workload": f"c2: first {len(scenes)} scenes, {n_air} air cells, {T} steps",
            "batched": batched, "plain": plain, "unit": UNIT, "ratio": batched / plain,
            "timing": "host wall clock around the runs (synchronize after each context's run)"}


def profile_run(args):
    """N direct-launch steps of the workload (its first --profile-scenes
    scenes), so that every kernel is a separate launch for ncu; prints the
    per-stage device times of 50 more steps."""
    import ard_gb300 as A
    n = args.profile
    cfg = workload(args.config, max(n, 64))
    scs = cfg["scenes"][:args.profile_scenes]
    h32 = float(np.float32(cfg["h"]))
    scenes = [A.build_scene(sc["air"], sc["sources"], sc["recorders"], h32, cfg["dt"], cfg["c0"], cfg["pml"])
              for sc in scs]
    sim = A.Simulation(scenes, max_steps=max(n, 64) * 4, use_graphs=False)
    load_series(sim, dict(cfg, scenes=scs), max(n, 64))
    sim.run(n)
    sim.synchronize()
    print(json.dumps({k: round(v * 1000, 1) for k, v in sim.profile(50).items()}), flush=True)
    sim.close()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--config", default="c4")
    ap.add_argument("--sim-steps", type=int, default=None, help="time steps per simulation (default: config)")
    ap.add_argument("--chunk", type=int, default=None,
                    help="time steps per benchmark step (default 1000 for runs of >= 10000 steps, else all)")
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-sample", type=int, default=1, help="minimum time steps of the CPU baseline sample")
    ap.add_argument("--cpu-seconds", type=float, default=10.0,
                    help="the CPU baseline steps on until this many seconds (within the series length)")
    ap.add_argument("--ref-sample", type=int, default=0,
                    help="time steps per reference-arm step (0: 1 for runs of >= 10000 steps, else 6)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--no-accuracy", action="store_true")
    ap.add_argument("--no-reference-arithmetic", action="store_true")
    ap.add_argument("--no-batching", action="store_true", help="skip the batched-against-plain measurement")
    ap.add_argument("--adjoint-steps", type=int, default=None,
                    help="steps of the adjoint measurement (default: the whole simulation)")
    ap.add_argument("--checkpoint-every", type=int, default=0,
                    help="adjoint checkpoint interval (0: the library's choice by free memory)")
    ap.add_argument("--plain", action="store_true", help="one context per scene, run one after another")
    ap.add_argument("--autotune", action="store_true", help="let ard_create time candidate layouts and keep the fastest")
    ap.add_argument("--profile", type=int, default=0,
                    help="profiling run for ncu: N direct-launch steps (no CUDA graphs, every kernel its own "
                         "launch), the per-stage times printed, no timing line")
    ap.add_argument("--profile-scenes", type=int, default=1, help="scenes of the profiling run")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3) if args.impl == "ours" else args.warmup

    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    local = int(os.environ.get("LOCAL_RANK", 0))
    if args.impl == "reference":
        return run_reference_arm(args, rank)
    if args.profile:
        return profile_run(args)

    import torch
    import ard_gb300 as A

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    cfg = workload(args.config, args.sim_steps, rank, world)
    S = cfg["steps"]
    chunk = min(args.chunk or default_chunk(S), S)
    h32 = float(np.float32(cfg["h"]))
    scenes = [A.build_scene(sc["air"], sc["sources"], sc["recorders"], h32, cfg["dt"], cfg["c0"], cfg["pml"])
              for sc in cfg["scenes"]]
    n_air = sum(s.air_cells for s in scenes)
    n_pml = sum(s.pml_cells for s in scenes)
    n_face = sum(s.face_cells for s in scenes)
    n_src = sum(len(sc["sources"]) for sc in cfg["scenes"])
    n_rec = sum(len(sc["recorders"]) for sc in cfg["scenes"])
    sims = ([A.Simulation([sc], max_steps=S, device=local, autotune=args.autotune) for sc in scenes]
            if args.plain else [A.Simulation(scenes, max_steps=S, device=local, autotune=args.autotune)])
    sim = sims[0]
    series = np.zeros((n_src, S), np.float32)
    k = 0
    for sc in cfg["scenes"]:
        for s in sc["series"]:
            series[k] = s[:S]
            k += 1
    src_off = np.cumsum([0] + [len(sc["sources"]) for sc in cfg["scenes"]]) if args.plain else [0, n_src]
    rec_off = np.cumsum([0] + [len(sc["recorders"]) for sc in cfg["scenes"]]) if args.plain else [0, n_rec]
    # pinned host buffers: the source samples of every benchmark step (contiguous per step) and
    # the recorder samples read back per step and context
    nchunks = (S + chunk - 1) // chunk
    pinned_src = torch.zeros((nchunks, n_src, chunk), dtype=torch.float32).pin_memory()
    for c in range(nchunks):
        n = min(chunk, S - c * chunk)
        pinned_src[c, :, :n] = torch.from_numpy(series[:, c * chunk:c * chunk + n])
    pinned_rec = [torch.empty((chunk, max(1, int(rec_off[i + 1] - rec_off[i]))), dtype=torch.float32).pin_memory()
                  for i in range(len(sims))]
    import ctypes as C
    fptr = lambda t: C.cast(t.data_ptr(), C.POINTER(C.c_float))
    stream = torch.cuda.Stream()
    handle = stream.cuda_stream
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")   # 256 MiB > 129 MB L2
    recorded = np.zeros((S, n_rec), np.float32)   # recorder samples of the timed simulation

    def bench_step(i, timed):
        """Benchmark step i: time steps [t0, t0 + n) of the current simulation,
        source upload and recorder read-back through the C ABI.  Returns the
        device milliseconds of the steps."""
        t0 = (i * chunk) % (nchunks * chunk)
        n = min(chunk, S - t0)
        c = t0 // chunk
        if t0 == 0:
            for sm in sims:
                sm.reset()
        for j, sm in enumerate(sims):
            if src_off[j + 1] > src_off[j]:
                sm._c(A.lib().ard_set_source_samples(sm._h, -1, -1, t0, n, fptr(pinned_src[c, int(src_off[j]):])))
        with torch.cuda.stream(stream):
            flush.fill_(1.0)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
        for sm in sims:
            sm.run(n, stream=handle)
        with torch.cuda.stream(stream):
            e1.record(stream)
        for j, sm in enumerate(sims):
            nr = int(rec_off[j + 1] - rec_off[j])
            if nr > 0:
                sm._c(A.lib().ard_read_recorders(sm._h, -1, fptr(pinned_rec[j]), t0, n))
                if timed:
                    recorded[t0:t0 + n, int(rec_off[j]):int(rec_off[j + 1])] = pinned_rec[j][:n, :nr].numpy()
        e1.synchronize()
        return e0.elapsed_time(e1), n

    for i in range(args.warmup):
        bench_step(i, False)
    torch.cuda.synchronize()
    for sm in sims:
        sm.reset()

    # ---- timed region: device time per step (value) and wall clock (e2e) ----
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    total_ms, total_steps = 0.0, 0
    w0 = time.perf_counter()
    for i in range(args.steps):
        ms, n = bench_step(i, True)
        total_ms += ms
        total_steps += n
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - w0
    clk = clocks.stop()
    if dist:
        t = torch.tensor([total_ms, e2e_s * 1e3], device="cuda", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms, e2e_s = float(t[0].item()), float(t[1].item()) / 1e3
        tot = torch.tensor([float(n_air)], device="cuda", dtype=torch.float64)
        dist.all_reduce(tot)
        n_air_all = float(tot.item())
    else:
        n_air_all = float(n_air)
    value = n_air_all * total_steps / (total_ms / 1e3) / 1e9
    ms_per_step = total_ms / args.steps
    fwd_s_per_time_step = total_ms / 1e3 / total_steps
    e2e = {"value": n_air_all * total_steps / e2e_s / 1e9, "unit": UNIT,
           "h2d_bytes_per_step": int(n_src * chunk * 4), "d2h_bytes_per_step": int(n_rec * chunk * 8)}

    # ---- per-stage device times (un-captured steps, CUDA events per kernel) ----
    sim.reset()
    with torch.cuda.stream(stream):
        flush.fill_(1.0)
    prof_steps = min(S, 200)
    stages = sim.profile(prof_steps, stream=handle)
    peak, peak_kind = peaks()
    prof_scenes = scenes[:1] if args.plain else scenes
    p_air = sum(s.air_cells for s in prof_scenes)
    p_pml = sum(s.pml_cells for s in prof_scenes)
    p_face = sum(s.face_cells for s in prof_scenes)
    modal_ms = stages[MODAL_STAGE]
    alg_bytes = BYTES_PER_AIR_CELL * p_air
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

    def hbm_stage(ms, nbytes):
        gbs = nbytes / (ms / 1e3) / 1e9 if ms > 0 else 0.0
        return {"ms": ms, "algorithmic_bytes": nbytes, "achieved_gbs": gbs, "frac": gbs / peak}

    f_ms = stages["fwd_rows"] + stages["fwd_cols"] + stages["inv_cols"] + stages["inv_rows"]
    flops = face_flops(prof_scenes)
    f_tf = flops / (f_ms / 1e3) / 1e12 if f_ms > 0 else 0.0
    tensor = "faces tensor-core" in sim.layout
    if tensor:
        # split TF32: three products per useful one, on the tensor cores
        tpk, tpk_src = tf32_peak_tflops()
        f_compute = {"path": "tcgen05 split TF32 (3 products per useful MAC)", "tensor_tflops": 3 * f_tf,
                     "tf32_peak_tflops": tpk, "tf32_peak_source": tpk_src, "frac_of_tf32_peak": 3 * f_tf / tpk}
    else:
        f_compute = {"path": "CUDA-core FP32", "fp32_fma_peak_tflops": FP32_FMA_TFLOPS,
                     "frac_of_fp32_fma_peak": f_tf / FP32_FMA_TFLOPS}
    f_bytes = face_bytes(prof_scenes)
    stage_roofline = {
        "modal": hbm_stage(modal_ms, BYTES_PER_AIR_CELL * p_air),
        "pml": hbm_stage(stages["pml"], BYTES_PER_PML_CELL * p_pml),
        "iface": hbm_stage(stages["iface"], BYTES_PER_FACE_CELL * p_face),
        "faces": dict({"ms": f_ms, "useful_flops": flops, "achieved_tflops": f_tf,
                       "algorithmic_bytes": f_bytes,
                       "achieved_gbs": f_bytes / (f_ms / 1e3) / 1e9 if f_ms > 0 else 0.0,
                       "frac_of_hbm": (f_bytes / (f_ms / 1e3) / 1e9 / peak) if f_ms > 0 else 0.0}, **f_compute),
        "recorder_and_sums": {"ms": stages["recorder"]},
        "peak_gbs": peak, "peak_source": peak_kind,
    }
    # whole step: the reference's per-step algorithmic bytes over the device time of one step
    step_bytes = BYTES_PER_AIR_CELL * n_air + BYTES_PER_PML_CELL * n_pml + BYTES_PER_FACE_CELL * n_face
    step_roofline = {"algorithmic_bytes_per_step": step_bytes, "ms_per_time_step": fwd_s_per_time_step * 1e3,
                     "achieved": step_bytes / fwd_s_per_time_step / 1e9, "unit": "GB/s",
                     "frac": step_bytes / fwd_s_per_time_step / 1e9 / peak}
    kps = sum(sm.kernels_per_step for sm in sims)
    launches = int(args.steps * (chunk * kps + (chunk // 32 + (1 if chunk % 32 else 0)) * len(sims)))
    layout = sim.layout
    for sm in sims:
        sm.close()

    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": describe(cfg, n_air, n_pml), "time_steps_per_step": chunk,
                       "simulation_steps": S,
                       "state": "carried across benchmark steps; the simulation restarts from rest at its length",
                       "scenes_per_rank": len(scenes),
                       "parallelism": ("plain: one context per scene, run one after another" if args.plain else
                                       "replicas" if len(cfg["scenes"]) == 1 else "scene shards"),
                       "l2": "flushed (256 MiB write) before every benchmark step",
                       "layout": layout},
            "roofline": roofline,
            "stage_roofline": stage_roofline,
            "step_roofline": step_roofline,
            "stage_ms_per_step": stages,
            "e2e": e2e,
            "gpu_launches": launches,
            "kernels_per_step": kps,
            "clocks": clk}

    # ---- the reference's FP32 arithmetic (the parity mode), shorter run ----
    rec_ref = None
    if not args.no_reference_arithmetic and not args.plain:
        rs = A.Simulation(scenes, max_steps=S, device=local, arithmetic=A.ARITH_REFERENCE)
        load_series(rs, cfg, S)
        n_ref = min(S, 2 * chunk)
        rs.run(min(S, chunk))
        rs.synchronize()
        rs.reset()
        with torch.cuda.stream(stream):
            flush.fill_(1.0)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
        rs.run(n_ref, stream=handle)
        with torch.cuda.stream(stream):
            e1.record(stream)
        e1.synchronize()
        rms = e0.elapsed_time(e1)
        rec_ref = rs.recorders(scene=-1, f64=True)
        rs.close()
        line["reference_arithmetic"] = {"value": n_air_all * n_ref / (rms / 1e3) / 1e9, "unit": UNIT,
                                        "time_steps": n_ref, "ms_per_time_step": rms / n_ref}
    if not args.no_accuracy and not args.plain:
        covered = min(S, args.steps * chunk)   # time steps the timed benchmark steps recorded
        line["accuracy"] = accuracy_measurement(A, cfg, scenes, local, rec32=recorded[:covered].astype(np.float64),
                                                rec_ref=rec_ref)
    if not args.no_adjoint and not args.plain:
        Sa = min(args.adjoint_steps or S, S)
        if args.steps * chunk >= Sa or Sa <= chunk:
            line["adjoint"] = adjoint_measurement(A, cfg, scenes, args, local, series, recorded[:Sa].copy(),
                                                  fwd_s_per_time_step)
    if not args.no_batching and not args.plain and rank == 0:
        line["batched_vs_plain"] = batching_measurement(A, local)
    if rank == 0 and not args.no_cpu_baseline:
        os.environ.setdefault("OMP_NUM_THREADS", str(os.cpu_count() or 1))
        line["cpu_baseline"] = cpu_baseline(cfg, args.cpu_sample, args.cpu_seconds)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
