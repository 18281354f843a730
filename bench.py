#!/usr/bin/env python
"""Benchmark: tracked frames/s of bi-objective (photometric + point-to-plane ICP,
lambda = 0.5) tracking at 640x480 with a 4-level pyramid over a 300-frame
seeded smooth trajectory, a keyframe every 10 frames, each keyframe fusing the
depth and colour of its 5 nearest tracked frames (the first five of its
segment) on the reconstruction stream.

One step tracks the whole trajectory: the 30 keyframe segments (keyframe 10j,
frames 10j+1 .. 10j+10 tracked against it, each frame starting from the
previous frame's pose as the reference tracker does between reference updates)
run as one batch of 30 tracker instances, so every launch serves all segments:
frames 1-5 of every segment, the fusion of those five frames into every
keyframe (second stream, poses and frames taken on the device), then frames
6-10 against the fused keyframes.

Pose error of every arm is measured against an FP64 oracle run of the same
trajectory (the same tracker, schedule and fusion with every operation in
double precision): a frame is tracked when its pose is within 1 mm / 0.05 deg
of the FP64 oracle's.

  value  frames/s tracked within the bound by the learned-init arm, inputs
         already in HBM (frames pre-rendered on the GPU), poses read back; the
         arm's raw frames/s and in-bound share are reported beside it
  e2e    the same through the C ABI from pinned host buffers: every step copies
         the frames host->device and the poses device->host inside the timed region

`--impl reference` times the reference algorithm's CPU implementation instead
(the oracle port, all host threads) on whole keyframe segments of the same
workload, fusion included.  Under torchrun each rank tracks its own trajectory
(weak scaling, no collective on the data path); rank 0 prints the JSON line.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

W, H, LEVELS = 640, 480, 4
N_FRAMES = 300
KEYFRAME_EVERY = 10
ITERS = (1, 3, 10, 5)
LAMBDA = 0.5
N_SELECT = 8192
# algorithmic bytes per point and GN iteration (photometric: xyz 12 + I_ref 4 +
# J 24 + 4 bilinear taps 16 + depth tap 4; the fused kernel keeps the residual
# and depth weight in registers, so the 16 bytes of the reference's separate
# passes are not counted; ICP: point+normal 24 + 4 taps x 12 + mask 4 + weight 4
# + index 4)
B_PHOTO = 60
B_ICP = 84
# learned initialisation: trained parameters and the shortened schedule it runs
LEARNED_WEIGHTS = "initnet_200k.npz"
# (in a sweep of shortened schedules on this trajectory: the most frames per
# second inside the pose bound among schedules that run every level and keep
# at least 90% of the frames in bound)
LEARNED_ITERS = (1, 2, 2, 1)
# the same rule for the plain start pose (the previous frame's): the fastest
# schedule that keeps 90% of the frames in bound
PLAIN_START_RULE_ITERS = (2, 2, 3, 1)
BOUND_MM, BOUND_DEG = 1.0, 0.05
# the settle rule (recon_batch_set_settle): a level ends once one iteration
# moves every translation entry by <= 0.1 mm and every rotation entry by
# <= 1e-4, the reference's schedule ITERS being the cap.  In a sweep on this
# trajectory with the previous frame's start pose (the FP32 oracle, which the
# GPU matches bit for bit) 0.05 / 0.1 / 0.2 mm kept 100% / 100% / 98.7% of the
# frames in bound at 12.8 / 10.7 / 8.8 executed iterations per frame (19 fixed)
SETTLE = (0.1, 1e-4)
# keyframe fusion: the first FUSE_FRAMES tracked frames of each segment, depth gate
FUSE_FRAMES = 5
GATE_MM = 30.0
# reconstruction stream: a 256^3 grid (134 MB) placed around the synthetic
# room, 30 depth frames with 0.1% depth noise (the update's 0.5%-of-cube
# consistency test rejects most pixels of noisier depth)
TSDF_R = 256
TSDF_FRAMES = 30
TSDF_CUBE = ((0.0, 150.0, -2350.0), (1750.0, 1750.0, 1750.0))
TSDF_NOISE = 0.001
METRIC = ("tracked frames/s at 640x480 (frames within 1mm/0.05deg of the FP64 oracle per second; frames outside "
          "the bound not counted): learned-init vs plain GPU")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--frames", type=int, default=N_FRAMES)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--plain-only", action="store_true", help="skip the learned-initialisation arm (profiling)")
    ap.add_argument("--no-tune", action="store_true", help="built-in tile shapes instead of the autotuner's")
    ap.add_argument("--no-batch", action="store_true", help="skip the 256-instance mixed-resolution workload")
    ap.add_argument("--no-mixed", action="store_true", help="skip the mixed-precision measurement")
    ap.add_argument("--batch-only", action="store_true", help="only the 256-instance workload (profiling)")
    ap.add_argument("--no-tsdf", action="store_true", help="skip the reconstruction-stream measurement")
    ap.add_argument("--tsdf-only", action="store_true", help="only the reconstruction-stream measurement")
    ap.add_argument("--tile", default=None, help="ICP chunks per CTA per level, e.g. 3,2,2,1 (no tuning)")
    return ap.parse_args()


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def rank_seed(rank: int) -> int:
    """Scene/trajectory seed of a rank: every rank tracks its own trajectory (weak scaling)."""
    return 1000 + 17 * rank


def max_over_ranks(x: float, world: int, device) -> float:
    """Slowest rank's time (the job finishes when the last rank does)."""
    if world <= 1:
        return float(x)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(world: int, frames_per_rank_step: int, steps: int, max_ms: float) -> float:
    """Frames/s of the whole job: all ranks' frames over the slowest rank's time."""
    return world * frames_per_rank_step * steps / (max_ms / 1000.0)


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock / throttle-reason samples during the timed region,
    kept in $RECON_BENCH_OUT (default bench_out/) as clocks_rank<i>.csv."""

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        out = os.environ.get("RECON_BENCH_OUT", os.path.join(ROOT, "bench_out"))
        self.path = os.path.join(out, f"clocks_rank{index}.csv")

    def __enter__(self):
        os.makedirs(os.path.dirname(self.path), exist_ok=True)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self):
        try:
            rows = [r.split(",") for r in open(self.path).read().strip().splitlines() if r.strip()]
        except Exception:
            rows = []
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        sm = [float(r[1]) for r in rows if r[1].strip().replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if r[2].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in rows:
            for k, nm in enumerate(names):
                if len(r) > 5 + k and r[5 + k].strip().lower() in ("active", "1"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(rows)}


# ---------------------------------------------------------------- workload
def make_workload(seed: int, n_frames: int):
    from recon_gb300 import synth
    cal = synth.make_calibration(W, H)
    scene = synth.make_scene(seed)
    poses = synth.smooth_trajectory(n_frames + 1, seed + 2)
    return cal, scene, poses


def render_frames_gpu(cal, scene, poses, seed, torch):
    import recon_gb300 as rg
    from recon_gb300 import synth
    n = len(poses)
    gray = torch.empty((n, H, W), dtype=torch.uint8, device="cuda")
    depth = torch.empty((n, H, W), dtype=torch.int16, device="cuda")
    for f in range(n):
        rg.render_depth(scene, synth.camera_struct(cal, "L", poses[f]), 0.01, seed + 1, f, depth[f])
        rg.render_gray(scene, synth.camera_struct(cal, "R", poses[f]), gray[f])
    torch.cuda.synchronize()
    return gray, depth


def segments(n_frames):
    """(keyframe index, [tracked frame indices]) per keyframe segment."""
    segs = []
    for k in range(0, n_frames, KEYFRAME_EVERY):
        segs.append((k, list(range(k + 1, min(k + KEYFRAME_EVERY, n_frames) + 1))))
    return segs


def make_batch(cal, n_inst, stream, precision=0):
    import recon_gb300 as rg
    cfg = rg.make_config(W, H, LEVELS, mode=rg.BIOBJECTIVE, iters=ITERS, n_select=N_SELECT, lam=LAMBDA,
                         precision=precision)
    return rg.Batch([cfg] * n_inst, [cal.calib] * n_inst, stream=stream)


def step_plan(segs):
    """The frame indices of one step: every segment's keyframe, and for each
    sequence position s frame s of every segment (a shorter segment repeats
    its last frame), with the mask of the positions that are its own frames."""
    steps = max(len(fr) for _, fr in segs)
    ref = np.array([k for k, _ in segs], np.int64)
    seq = np.array([[fr[min(s, len(fr) - 1)] for _, fr in segs] for s in range(steps)], np.int64)
    own = np.array([[s < len(fr) for _, fr in segs] for s in range(steps)])
    return ref, seq, own


def run_step(batch, plan, gray_src, depth_src, poses_out):
    """Tracks every segment of the trajectory once (inputs: frame stacks
    [frames, H, W] on the device or in pinned host memory).

    The keyframes of all segments are set in one call; the segments' first
    FUSE_FRAMES frames are tracked as one sequence (recon_batch_track_sequence:
    frame s of every segment per launch, each starting from the previous
    frame's pose), fused into the keyframes on the reconstruction stream from
    the device (recon_batch_fuse_sequence: depth and colour, tracked poses),
    and the remaining frames are tracked against the fused keyframes."""
    ref, seq, own = plan
    batch.set_reference_frames(gray_src, depth_src, ref)
    T1, _ = batch.track_sequence_frames(gray_src, depth_src, seq[:FUSE_FRAMES])
    batch.fuse_sequence(FUSE_FRAMES, GATE_MM)
    T2, _ = batch.track_sequence_frames(gray_src, depth_src, seq[FUSE_FRAMES:])
    T = np.concatenate([T1, T2])
    poses_out[seq[own]] = T[own]
    return poses_out


# ---------------------------------------------------------------- CPU side
def cpu_track(cal, gray_np, depth_np, segs_sel, threads):
    """The FP32 oracle (CPU port of the reference algorithm, plain schedule)
    tracking whole keyframe segments as the GPU step does: keyframe, the first
    FUSE_FRAMES frames, depth/colour fusion of those frames, the rest.
    Returns (frames/s, poses {frame: T}, frames, seconds)."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_lib as O
    O.lib().orc_set_threads(threads)
    cfg = O.make_config(W, H, LEVELS, mode=O.BIOBJECTIVE, iters=ITERS, n_select=N_SELECT, lam=LAMBDA)
    out = {}
    n = 0
    t0 = time.perf_counter()
    for k, fr in segs_sel:
        orc = O.OracleTracker(cfg, cal.calib)
        orc.set_reference(gray_np[k], depth_np[k])
        T, Ts = None, []
        for s, f in enumerate(fr):
            if s == FUSE_FRAMES:
                orc.fuse_keyframe([depth_np[x] for x in fr[:FUSE_FRAMES]], np.stack(Ts), gate=GATE_MM,
                                  grays=[gray_np[x] for x in fr[:FUSE_FRAMES]])
            orc.set_current(gray_np[f], depth_np[f])
            T, _ = orc.track(T)
            Ts.append(T.copy())
            out[f] = T.copy()
            n += 1
        orc.close()
    dt = time.perf_counter() - t0
    O.lib().orc_set_threads(0)
    return n / dt, out, n, dt


def fp64_trajectory(cal, gray_np, depth_np, segs, iters=ITERS, mode=None, lam=LAMBDA, levels=LEVELS, width=W,
                    height=H, n_select=N_SELECT, fuse=True):
    """The FP64 oracle over the trajectory: every segment as the GPU step
    tracks it (keyframe, FUSE_FRAMES frames, depth/colour fusion with the FP64
    poses, the rest), every operation in double.  Returns ({frame: T64}, s)."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_lib as O
    O.lib().orc_set_threads(0)
    cfg = O.make_config(width, height, levels, mode=O.BIOBJECTIVE if mode is None else mode, iters=iters,
                        n_select=n_select, lam=lam)
    out = {}
    t0 = time.perf_counter()
    for k, fr in segs:
        orc = O.Oracle64Tracker(cfg, cal.calib)
        orc.set_reference(gray_np[k], depth_np[k])
        T, Ts = None, []
        for s, f in enumerate(fr):
            if fuse and s == FUSE_FRAMES:
                orc.fuse_keyframe([depth_np[x] for x in fr[:FUSE_FRAMES]], np.stack(Ts), gate=GATE_MM,
                                  grays=[gray_np[x] for x in fr[:FUSE_FRAMES]])
            orc.set_current(gray_np[f], depth_np[f])
            T = orc.track(T)
            Ts.append(T.copy())
            out[f] = T.copy()
        orc.close()
    return out, time.perf_counter() - t0


def host_frames(cal, scene, poses, seed, frames):
    """Renders the given frames on the CPU twin (identical to the GPU renderer)."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_lib as O
    from recon_gb300 import synth
    g, d = {}, {}
    for f in frames:
        g[f], d[f] = O.render_pair(scene, synth.camera_struct(cal, "L", poses[f]),
                                   synth.camera_struct(cal, "R", poses[f]), noise_rel=0.01,
                                   noise_seed=seed + 1, frame=f)
    return g, d


def reference_arm(args, rank, world):
    if rank != 0:
        return 0
    seed = 1000
    cal, scene, poses = make_workload(seed, args.frames)
    segs = segments(args.frames)
    threads = os.cpu_count() or 1
    sample_segs = segs[:1]
    need = sorted({k for k, _ in sample_segs} | {f for _, fr in sample_segs for f in fr})
    g, d = host_frames(cal, scene, poses, seed, need)
    times = []
    nseg = 0
    for i in range(args.warmup + args.steps):
        fps, _, n, dt = cpu_track(cal, g, d, sample_segs, threads)
        nseg = n
        if i >= args.warmup:
            times.append(dt / n)
    fps = 1.0 / float(np.mean(times))
    sample = (f"one keyframe segment per step ({nseg} frames tracked, the first {FUSE_FRAMES} fused into the "
              f"keyframe), plain schedule {'/'.join(map(str, ITERS))}, all {threads} host threads")
    line = {
        "impl": "reference", "metric": METRIC,
        "value": fps, "unit": "frames/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * float(np.mean(times)) * nseg, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "fp32", "data": "synthetic",
        "config": {"workload": "bi-objective lambda=0.5, 640x480, 4 levels, 8192 photometric points, keyframe every "
                               "10 frames, each keyframe fusing the depth and colour of its first 5 tracked frames",
                   "schedule": list(ITERS),
                   "method": "the reference's own tracker (previous-frame start, its schedule); every frame is "
                             "within the bound of the FP64 oracle (FP32 vs FP64 difference only)",
                   "sample_per_step": sample},
        "cpu_baseline": {"value": fps, "unit": "frames/s", "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": fps, "unit": "frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------- main
def load_net_params():
    """Trained parameters of the learned initialisation (recon_gb300/weights), or None."""
    path = os.path.join(ROOT, "recon_gb300", "weights", LEARNED_WEIGHTS)
    if not os.path.exists(path):
        return None, None
    z = np.load(path)
    return z["params"], {"file": os.path.relpath(path, ROOT), "pairs": int(z["pairs"]), "epochs": int(z["epochs"]),
                         "validation_start_error_median": {"deg": float(z["val_rot_deg_median"]),
                                                           "mm": float(z["val_trans_mm_median"])}}


def pose_errors(a, b, frames):
    from recon_gb300 import synth
    return np.array([synth.pose_error(np.asarray(a[f], np.float64), np.asarray(b[f], np.float64)) for f in frames])


def error_summary(e):
    ok = (e[:, 0] <= BOUND_MM) & (e[:, 1] <= BOUND_DEG)
    return {"within_bound": float(ok.mean()), "frames": int(len(ok)), "out_of_bound": int((~ok).sum()),
            "median_mm": float(np.median(e[:, 0])), "p99_mm": float(np.percentile(e[:, 0], 99)),
            "max_mm": float(e[:, 0].max()), "median_deg": float(np.median(e[:, 1])),
            "p99_deg": float(np.percentile(e[:, 1], 99)), "max_deg": float(e[:, 1].max())}, ok


# ---------------------------------------------------------------- batched workload
BATCH_N = 256
BATCH_RES = [(80, 60), (160, 120), (320, 240), (640, 480)]


def batch_workload(seed: int, torch):
    """The batched-tracking workload: 256 instances whose resolutions are drawn
    uniformly from 80x60 / 160x120 / 320x240 / 640x480 (4 levels at 640, else 3),
    each a seeded scene rendered at the identity and at a start offset of
    0.5-4 deg about a random axis and 0.5-50 mm along a random direction,
    4-12 Gauss-Newton iterations per level drawn per instance, and
    N_sel = min(8192, floor(W*H/2/1024)*1024)."""
    import recon_gb300 as rg
    from recon_gb300 import synth
    rng = np.random.default_rng(seed)
    cals = {r: synth.make_calibration(*r) for r in BATCH_RES}
    inst = []
    for i in range(BATCH_N):
        Wi, Hi = BATCH_RES[int(rng.integers(len(BATCH_RES)))]
        L = 4 if Wi == 640 else 3
        iters = tuple(int(v) for v in rng.integers(4, 13, size=L))
        P = int(min(8192, (Wi * Hi // 2 // 1024) * 1024))
        deg, mm = float(rng.uniform(0.5, 4.0)), float(rng.uniform(0.5, 50.0))
        Tcur = synth.offset_pose(int(rng.integers(1 << 30)), deg, mm)
        scene = synth.make_scene(int(rng.integers(1 << 30)))
        cal = cals[(Wi, Hi)]
        g = torch.empty((2, Hi, Wi), dtype=torch.uint8, device="cuda")
        d = torch.empty((2, Hi, Wi), dtype=torch.int16, device="cuda")
        for f, T in enumerate((np.eye(4), Tcur)):
            rg.render_depth(scene, synth.camera_struct(cal, "L", T), 0.01, seed + 1, f, d[f])
            rg.render_gray(scene, synth.camera_struct(cal, "R", T), g[f])
        inst.append({"W": Wi, "H": Hi, "L": L, "iters": iters, "P": P, "cal": cal, "scene": scene, "Tcur": Tcur,
                     "gt": synth.relative_pose(np.eye(4), Tcur), "g": g, "d": d,
                     "cfg": rg.make_config(Wi, Hi, L, mode=rg.BIOBJECTIVE, iters=iters, n_select=P, lam=LAMBDA)})
    torch.cuda.synchronize()
    return inst


def batch_arm(args, torch, world, rank, seed):
    """Tracks the batched workload: one step tracks all 256 instances from the
    identity (one graph replay of the whole per-level schedule).  Returns the
    throughput, accuracy against the rendering poses, the per-kernel times and
    the linearisation kernel's roofline."""
    import recon_gb300 as rg
    from recon_gb300 import synth
    from recon_gb300.tune import autotune_icp_chunks
    inst = batch_workload(seed, torch)
    stream = torch.cuda.Stream()
    b = rg.Batch([x["cfg"] for x in inst], [x["cal"].calib for x in inst], stream=stream.cuda_stream)
    b.set_reference([x["g"][0] for x in inst], [x["d"][0] for x in inst])
    b.set_current([x["g"][1] for x in inst], [x["d"][1] for x in inst])
    T0 = np.tile(np.eye(4, dtype=np.float32), (BATCH_N, 1, 1))
    if args.tile:
        b.set_icp_chunks_per_cta([int(v) for v in args.tile.split(",")])
        chosen = b.icp_chunks_per_cta()
    else:
        chosen, _ = autotune_icp_chunks(b, T_init=T0)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    for _ in range(args.warmup):
        b.track_async(T0)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    e0.record(stream)
    for _ in range(args.steps):
        b.track_async(T0)
    e1.record(stream)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    ms = max_over_ranks(e0.elapsed_time(e1), world, "cuda")
    T, stats = b.poses()
    err = np.array([synth.pose_error(T[i].astype(np.float64), inst[i]["gt"]) for i in range(BATCH_N)])
    # per-kernel event timing and the work counters over the same K steps
    b.enable_timing(True)
    b.work(reset=True)
    b.timing(reset=True)
    for _ in range(args.steps):
        b.track_async(T0)
    torch.cuda.synchronize()
    timing = b.timing(reset=True)
    work = b.work(reset=True).astype(np.float64)
    b.enable_timing(False)
    it_ms, it_launches = timing["gn_iteration"]
    bytes_iter = float(work[:, 0].sum() * B_PHOTO + work[:, 1].sum() * B_ICP)
    peak, peak_kind = load_peaks()
    achieved = bytes_iter / (it_ms / 1000.0) / 1e9 if it_ms > 0 else 0.0
    pix = sum(x["W"] * x["H"] for x in inst)
    out = {"workload": "256 instances, resolutions uniform over 80x60/160x120/320x240/640x480, bi-objective "
                       "lambda=0.5, start offsets 0.5-4 deg / 0.5-50 mm, 4-12 iterations per level, "
                       "N_sel=min(8192, floor(W*H/2/1024)*1024)",
           "resolution_counts": {f"{w}x{h}": sum(1 for x in inst if x["W"] == w) for w, h in BATCH_RES},
           "level0_pixels": pix, "gn_iterations": int(sum(sum(x["iters"]) for x in inst)),
           "tracked_frames_per_s": world * BATCH_N * args.steps / (ms / 1000.0), "ms_per_step": ms / args.steps,
           "tile": chosen[:4],
           "vs_ground_truth": {"median_mm": float(np.median(err[:, 0])), "median_deg": float(np.median(err[:, 1])),
                               "within_5mm_0.5deg": float(np.mean((err[:, 0] <= 5.0) & (err[:, 1] <= 0.5)))},
           "kernel_ms_per_step": {k: v[0] / args.steps for k, v in timing.items() if v[1]},
           "roofline_k_iter": {"achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                               "peak_source": peak_kind, "launches_per_step": it_launches / args.steps}}
    if rank == 0 and not args.no_cpu:
        out["pose_error_vs_oracle"] = batch_oracle_check(inst, T)
    b.close()
    return out


def batch_oracle_check(inst, T):
    """One instance of each resolution tracked by the oracle from CPU-rendered
    copies of the same frames; returns the largest pose difference."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_lib as O
    worst, checked = 0.0, []
    for w, h in BATCH_RES:
        i = next((k for k, x in enumerate(inst) if x["W"] == w), None)
        if i is None:
            continue
        x = inst[i]
        g0, d0 = x["g"][0].cpu().numpy(), x["d"][0].cpu().numpy()
        g1, d1 = x["g"][1].cpu().numpy(), x["d"][1].cpu().numpy()
        orc = O.OracleTracker(O.make_config(w, h, x["L"], mode=O.BIOBJECTIVE, iters=x["iters"], n_select=x["P"],
                                            lam=LAMBDA), x["cal"].calib)
        orc.set_reference(g0, d0.view(np.uint16))
        orc.set_current(g1, d1.view(np.uint16))
        To, _ = orc.track()
        orc.close()
        worst = max(worst, float(np.abs(To - T[i]).max()))
        checked.append(i)
    return {"instances": checked, "max_abs_pose_diff": worst, "bit_identical": worst == 0.0}


def profiled_traffic():
    """DRAM bytes per average k_iter launch of this workload, from the committed
    ncu summary (profiles/k_iter_640x480_biobj_30inst.md), or None."""
    path = os.path.join(ROOT, "profiles", "k_iter_640x480_biobj_30inst.md")
    try:
        for line in open(path):
            if line.startswith("traffic_bytes_per_launch:"):
                return float(line.split(":")[1])
    except (OSError, ValueError):
        pass
    return None


def config1_arm(args, torch, seed=2024):
    """Config 1: one 320x240 frame pair (2 deg / 20 mm offset about a random
    axis), photometric, 3 levels, 10 Gauss-Newton iterations per level,
    256-bin MAD histogram, FP32.  GPU: one tracker instance, frames resident,
    K timed tracking runs from the identity (CUDA events); CPU: the oracle port
    at 1 thread and at all threads on the same pair; pose error against the
    FP64 oracle."""
    import recon_gb300 as rg
    from recon_gb300 import synth
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_lib as O
    Wc, Hc, Lc, it = 320, 240, 3, (10, 10, 10)
    cal = synth.make_calibration(Wc, Hc)
    sc = synth.make_scene(seed)
    Tcur = synth.offset_pose(seed + 1, 2.0, 20.0)
    g0, d0 = O.render_pair(sc, synth.camera_struct(cal, "L", np.eye(4)), synth.camera_struct(cal, "R", np.eye(4)),
                           noise_rel=0.01, noise_seed=seed + 2, frame=0)
    g1, d1 = O.render_pair(sc, synth.camera_struct(cal, "L", Tcur), synth.camera_struct(cal, "R", Tcur),
                           noise_rel=0.01, noise_seed=seed + 2, frame=1)
    cfg = rg.make_config(Wc, Hc, Lc, mode=rg.PHOTOMETRIC, iters=it, hist_bins=256)
    trk = rg.Tracker(cfg, cal.calib)
    dev = [torch.from_numpy(x).cuda() for x in (g0, d0.view(np.int16), g1, d1.view(np.int16))]
    trk.set_reference(dev[0], dev[1])
    trk.set_current(dev[2], dev[3])
    I = np.eye(4, dtype=np.float32).reshape(1, 16)
    st = torch.cuda.ExternalStream(trk.stream())
    for _ in range(args.warmup):
        trk.track_async(I)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = max(args.steps, 1) * 20
    e0.record(st)
    for _ in range(reps):
        trk.track_async(I)
    e1.record(st)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    T, _ = trk.poses()
    trk.close()
    ocfg = O.make_config(Wc, Hc, Lc, mode=O.PHOTOMETRIC, iters=it, hist_bins=256)
    cpu = {}
    for threads in (1, os.cpu_count() or 1):
        O.lib().orc_set_threads(threads)
        orc = O.OracleTracker(ocfg, cal.calib)
        orc.set_reference(g0, d0)
        orc.set_current(g1, d1)
        n, t0 = 0, time.perf_counter()
        while n < 3 or time.perf_counter() - t0 < 2.0:
            To, _ = orc.track(np.eye(4, dtype=np.float32))
            n += 1
        cpu[threads] = n / (time.perf_counter() - t0)
        orc.close()
    O.lib().orc_set_threads(0)
    o64 = O.Oracle64Tracker(ocfg, cal.calib)
    o64.set_reference(g0, d0)
    o64.set_current(g1, d1)
    T64 = o64.track(np.eye(4))
    o64.close()
    mm, deg = synth.pose_error(T[0].astype(np.float64), T64)
    gmm, gdeg = synth.pose_error(T64, synth.relative_pose(np.eye(4), Tcur))
    return {"workload": "one 320x240 frame pair, 2 deg / 20 mm offset, photometric, 3 levels, iterations 10/10/10, "
                        "256-bin MAD histogram, FP32",
            "gpu_pairs_per_s": 1000.0 / ms, "gpu_ms_per_pair": ms,
            "gpu_timing": f"{reps} tracking runs from the identity on one instance, CUDA events, frames resident",
            "cpu_pairs_per_s": {"1_thread": cpu[1], f"{os.cpu_count() or 1}_threads": cpu[os.cpu_count() or 1]},
            "gpu_bit_identical_to_cpu_port": bool(np.array_equal(T[0].view(np.uint32), To.view(np.uint32))),
            "vs_fp64_oracle": {"mm": mm, "deg": deg},
            "fp64_vs_rendering_pose": {"mm": gmm, "deg": gdeg}}


def tsdf_arm(args, torch, seed=77):
    """Reconstruction stream (VoxelGrid): TSDF_FRAMES depth frames (640x480,
    rendered on the GPU) fused into a TSDF_R^3 grid, each followed by a ray
    cast and shading from its pose.  One step = reset + the whole sequence.
    Per-kernel CUDA-event timing in a separate pass with an L2 flush (a 256 MB
    write) before every update; algorithmic bytes of an update from its voxel
    counts; grid and last ray cast checked bit for bit against the CPU oracle
    on the first frames; the oracle's update and ray cast timed on the host."""
    import recon_gb300 as rg
    from recon_gb300 import synth
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_lib as O
    cal = synth.make_calibration(W, H)
    scene = synth.make_scene(seed)
    poses = synth.smooth_trajectory(TSDF_FRAMES, seed + 2).astype(np.float32)
    depth = torch.empty((TSDF_FRAMES, H, W), dtype=torch.int16, device="cuda")
    for f in range(TSDF_FRAMES):
        rg.render_depth(scene, synth.camera_struct(cal, "L", poses[f]), TSDF_NOISE, seed + 1, f, depth[f])
    torch.cuda.synchronize()
    K = rg.normalized_K(cal.camera_K("L"), W, H)
    origin, dim = TSDF_CUBE
    prm = rg.tsdf_params(TSDF_R, W, H, cal.min_dist, cal.max_dist, cube_origin=origin, cube_dim=dim)
    v = rg.TSDF(prm)
    st = torch.cuda.ExternalStream(v.stream())

    def sweep(n=TSDF_FRAMES, flush=None):
        v.reset()
        for f in range(n):
            v.set_dist_depth16(depth[f])
            if flush is not None:
                with torch.cuda.stream(st):
                    flush.fill_(f)
            v.update(poses[f], K)
            v.raycast(poses[f], K)

    for _ in range(max(args.warmup, 1)):
        sweep()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launches0 = rg.launch_count()
    e0.record(st)
    for _ in range(args.steps):
        sweep()
    e1.record(st)
    torch.cuda.synchronize()
    ms_step = e0.elapsed_time(e1) / args.steps
    launches = (rg.launch_count() - launches0) / args.steps
    # per-kernel timing, cold L2 before each update
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    v.enable_timing(True)
    v.timing(reset=True)
    for _ in range(args.steps):
        sweep(flush=flush)
    tm = v.timing(reset=True)
    v.enable_timing(False)
    del flush
    # voxel counts of the same sweep (untimed)
    v.enable_counting(True)
    v.counts(reset=True)
    sweep()
    cnt = v.counts(reset=True).astype(np.float64)
    v.enable_counting(False)
    upd_ms, upd_n = tm["update"]
    per_upd_ms = upd_ms / max(upd_n, 1)
    nvox = float(TSDF_R) ** 3
    dist_bytes = W * H * 4
    alg_bytes = (8.0 * cnt[1] + 8.0 * cnt[2]) / TSDF_FRAMES + dist_bytes
    ref_bytes = 16.0 * cnt[1] / TSDF_FRAMES + dist_bytes
    achieved = alg_bytes / (per_upd_ms / 1000.0) / 1e9
    peak, peak_kind = load_peaks()
    rc_ms, rc_n = tm["raycast"]
    sh_ms, sh_n = tm["shading"]
    # parity on the first frames against the CPU oracle (the checker)
    n_chk = 6
    sweep(n_chk)
    g_gpu = v.get("tsdf")
    xyz_gpu = v.get("xyz")
    op = O.tsdf_params(TSDF_R, W, H, cal.min_dist, cal.max_dist, origin=origin, dim=dim)
    o = O.OracleTSDF(op)
    dh = depth[:n_chk].cpu().numpy().view(np.uint16)
    threads = os.cpu_count() or 1
    O.lib().orc_set_threads(threads)
    t_upd, t_ray = [], []
    for f in range(n_chk):
        t0 = time.perf_counter()
        o.update(dh[f].astype(np.float32), poses[f], K)
        t1 = time.perf_counter()
        xyz_o = o.raycast(poses[f], K)
        t_ray.append(time.perf_counter() - t1)
        t_upd.append(t1 - t0)
    same_grid = bool(np.array_equal(g_gpu.view(np.uint32), o.grid.view(np.uint32)))
    same_xyz = bool(np.array_equal(xyz_gpu.view(np.uint32), xyz_o.view(np.uint32)))
    O.lib().orc_set_threads(1)
    t0 = time.perf_counter()
    o.update(dh[0].astype(np.float32), poses[0], K)
    t_upd1 = time.perf_counter() - t0
    O.lib().orc_set_threads(0)
    hits = float((xyz_gpu[3::4] > 0).mean())
    v.close()
    return {
        "workload": f"{TSDF_R}^3 float2 grid ({int(nvox * 8) >> 20} MB, cube centre {origin} half-size {dim[0]} mm), "
                    f"{TSDF_FRAMES} depth frames 640x480 ({TSDF_NOISE * 100:.1f}% depth noise) along a smooth "
                    f"trajectory; per frame: distance map, update, ray cast (3 refinement steps) and shading",
        "frames_per_s": 1000.0 * TSDF_FRAMES / (ms_step / 1.0) if ms_step > 0 else None,
        "ms_per_step": ms_step, "gpu_launches_per_step": launches,
        "update": {"ms_per_launch": per_upd_ms, "voxels_per_s": nvox / (per_upd_ms / 1000.0),
                   "voxels_projected_per_update": cnt[0] / TSDF_FRAMES,
                   "voxels_fused_per_update": cnt[1] / TSDF_FRAMES,
                   "voxels_changed_per_update": cnt[2] / TSDF_FRAMES,
                   "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                                "frac": achieved / peak, "peak_source": peak_kind,
                                "algorithmic_bytes_per_launch": alg_bytes,
                                "bytes_rule": "8 B read per fused voxel + 8 B written per changed voxel + the "
                                              "distance map (4 B per pixel)",
                                "reference_kernel_bytes_per_launch": ref_bytes,
                                "timing": "CUDA events around each update launch, L2 flushed before it"}},
        "raycast": {"ms_per_launch": rc_ms / max(rc_n, 1), "rays_per_s": W * H / (rc_ms / max(rc_n, 1) / 1000.0),
                    "hit_share": hits, "shading_ms_per_launch": sh_ms / max(sh_n, 1)},
        "kernel_ms": {k: val[0] for k, val in tm.items()},
        "kernel_launches": {k: val[1] for k, val in tm.items()},
        "parity": {"frames": n_chk, "grid_bit_identical_to_oracle": same_grid,
                   "raycast_bit_identical_to_oracle": same_xyz},
        "cpu_baseline": {"kind": "port", "cores": threads,
                         "update_ms": 1000.0 * float(np.median(t_upd)), "raycast_ms": 1000.0 * float(np.median(t_ray)),
                         "update_ms_1_thread": 1000.0 * t_upd1,
                         "frames_per_s": 1.0 / (float(np.median(t_upd)) + float(np.median(t_ray))),
                         "sample": f"the oracle's update and ray cast of the first {n_chk} frames "
                                   f"({threads} OpenMP threads; one update at 1 thread)"},
    }


def kinect_arm(args, torch, seed=91, frames=30):
    """Kinect pre-processing (multicore.cpp routines) on the GPU: per frame the
    disparity -> depth conversion (full resolution, the (-4, -3) shift), RGB ->
    gray and the gray undistortion of a 640x480 frame, device buffers, CUDA
    events on torch's stream; the oracle's per-frame time beside it and the
    last frame checked bit for bit against it."""
    import recon_gb300 as rg
    from recon_gb300 import synth
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_lib as O
    rng = np.random.default_rng(seed)
    cal = synth.make_calibration(W, H, distortion=True)
    c0, c1 = float(cal.calib[61]), float(cal.calib[42])
    disp = rng.integers(280, 1040, (frames, H, W)).astype(np.uint16)
    disp[rng.random((frames, H, W)) < 0.05] = 2047
    rgb = rng.integers(0, 256, (frames, H, W, 3)).astype(np.uint8)
    K = np.ascontiguousarray(cal.calib[0:9], np.float32)
    iK = np.ascontiguousarray(cal.calib[9:18], np.float32)
    kc = np.ascontiguousarray(cal.calib[18:23], np.float32)
    d_disp = torch.from_numpy(disp.view(np.int16)).cuda()
    d_rgb = torch.from_numpy(rgb).cuda()
    z = torch.empty((frames, H, W), dtype=torch.float32, device="cuda")
    gray = torch.zeros((frames, H, W), dtype=torch.uint8, device="cuda")
    und = torch.zeros((frames, H, W), dtype=torch.uint8, device="cuda")

    def step():
        for f in range(frames):
            rg.kinect_disparity_to_depth(d_disp[f], c0, c1, cal.min_dist, cal.max_dist, -4.0, -3.0, out=z[f])
            rg.kinect_rgb_to_gray(d_rgb[f], out=gray[f])
            rg.kinect_undistort_gray(gray[f], K, iK, kc, out=und[f])

    def graph_ms(fn):
        """ms per frame of fn's launches for all frames, captured once as a CUDA
        graph and replayed, so that the time is the device's and not the
        Python loop's"""
        for _ in range(max(args.warmup, 1)):
            fn()
        torch.cuda.synchronize()
        graph = torch.cuda.CUDAGraph()
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):
            with torch.cuda.graph(graph):
                fn()
        torch.cuda.synchronize()
        for _ in range(max(args.warmup, 1)):
            graph.replay()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(args.steps):
            graph.replay()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / args.steps / frames

    ms = graph_ms(step)
    # the reference's GPU capture path (capture/VideoPreProcessorGPU.cpp):
    # disparity as float -> normalised half-resolution depth, RGB -> float RGB
    # -> float gray
    disp_fl = torch.empty((frames, H, W), dtype=torch.float32, device="cuda")
    zlow = torch.empty((frames, H // 2, W // 2), dtype=torch.float32, device="cuda")
    rgbh = torch.empty((frames, H, W, 3), dtype=torch.float32, device="cuda")
    grayh = torch.empty((frames, H, W), dtype=torch.float32, device="cuda")

    def step_gpu_path():
        for f in range(frames):
            rg.kinect_disparity_to_float(d_disp[f], out=disp_fl[f])
            rg.kinect_depth_normalized(disp_fl[f], c0, c1, cal.min_dist, cal.max_dist, -4.0, -3.0, out=zlow[f])
            rg.kinect_rgb_to_hdr(d_rgb[f], out=rgbh[f])
            rg.kinect_rgb_to_gray_hdr(rgbh[f], out=grayh[f])

    ms_gpu_path = graph_ms(step_gpu_path)
    # the oracle on the last frame (and its time per frame, one thread)
    f = frames - 1
    t0 = time.perf_counter()
    zo = np.zeros((H, W), np.float32)
    dispf = np.ascontiguousarray(disp[f])
    O.lib().orc_kinect_d2z(O.ptr(dispf), W, H, c0, c1, cal.min_dist, cal.max_dist, -4.0, -3.0, O.ptr(zo))
    go = np.zeros((H, W), np.uint8)
    rgbf = np.ascontiguousarray(rgb[f])
    O.lib().orc_kinect_rgb2gray(O.ptr(rgbf), W, H, O.ptr(go))
    uo = np.zeros((H, W), np.uint8)
    O.lib().orc_kinect_undistort(O.ptr(go), W, H, O.ptr(K), O.ptr(iK), O.ptr(kc), O.ptr(uo))
    cpu_ms = 1000.0 * (time.perf_counter() - t0)
    same = (np.array_equal(z[f].cpu().numpy().view(np.uint32), zo.view(np.uint32))
            and np.array_equal(gray[f].cpu().numpy(), go) and np.array_equal(und[f].cpu().numpy(), uo))
    n = W * H
    t0 = time.perf_counter()
    uo = np.zeros((H, W), np.float32)
    disp_last = np.ascontiguousarray(disp[f])
    O.lib().orc_kinect_disparity_to_float(O.ptr(disp_last), n, O.ptr(uo))
    zlo = np.zeros((H // 2, W // 2), np.float32)
    O.lib().orc_kinect_depth_normalized(None, O.ptr(uo), W, H, c0, c1, cal.min_dist, cal.max_dist, -4.0, -3.0,
                                        O.ptr(zlo))
    ho = np.zeros((H, W, 3), np.float32)
    O.lib().orc_kinect_rgb_to_hdr(O.ptr(rgbf), n, O.ptr(ho))
    gho = np.zeros((H, W), np.float32)
    O.lib().orc_kinect_rgb_hdr_to_gray(O.ptr(ho), n, O.ptr(gho))
    cpu_ms_gpu_path = 1000.0 * (time.perf_counter() - t0)
    same_gpu_path = all(np.array_equal(a.cpu().numpy().view(np.uint32), b.view(np.uint32))
                        for a, b in ((disp_fl[f], uo), (zlow[f], zlo), (rgbh[f], ho), (grayh[f], gho)))
    return {"workload": f"{frames} frames of 640x480: 11-bit disparity -> depth (shift -4, -3), RGB -> gray, gray "
                        "undistortion (radial), device buffers, the step's launches replayed as a CUDA graph",
            "frames_per_s": 1000.0 / ms, "us_per_frame": 1000.0 * ms,
            "bytes_per_frame": W * H * (2 + 4 + 3 + 1 + 1 + 1),
            "bit_identical_to_oracle": bool(same),
            "cpu_baseline": {"kind": "port", "cores": 1, "ms_per_frame": cpu_ms,
                             "sample": "the oracle's three routines on one frame, one thread"},
            "gpu_capture_path": {
                "workload": f"{frames} frames of 640x480 through the reference's GPU capture kernels: disparity as "
                            "float -> normalised 320x240 depth (shift -4, -3), RGB -> float RGB -> float gray, "
                            "device buffers, graph-replayed",
                "frames_per_s": 1000.0 / ms_gpu_path, "us_per_frame": 1000.0 * ms_gpu_path,
                "bytes_per_frame": W * H * (2 + 4 + 4 + 1 + 3 + 12 + 12 + 4),
                "bit_identical_to_oracle": bool(same_gpu_path),
                "cpu_baseline": {"kind": "port", "cores": 1, "ms_per_frame": cpu_ms_gpu_path,
                                 "sample": "the oracle's four steps on one frame, one thread"}}}


def main():
    args = parse()
    rank, world, local = dist_info()
    if args.impl == "reference":
        return reference_arm(args, rank, world)
    import torch
    import recon_gb300 as rg
    from recon_gb300 import synth
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    seed = rank_seed(rank)
    if args.tsdf_only:
        out = tsdf_arm(args, torch)
        kin = kinect_arm(args, torch)
        if rank == 0:
            print(json.dumps({"metric": "reconstruction frames/s (TSDF update + ray cast), 256^3 grid, 640x480",
                              "unit": "frames/s", "value": out["frames_per_s"], "n_gpus": world,
                              "steps": args.steps, "warmup": args.warmup, "tsdf": out,
                              "kinect_preprocessing": kin}), flush=True)
        if world > 1:
            torch.distributed.destroy_process_group()
        return 0
    if args.batch_only:
        out = batch_arm(args, torch, world, rank, 5000 + 7919 * rank)
        if rank == 0:
            print(json.dumps({"metric": "tracked frames/s, 256-instance mixed-resolution batch", "unit": "frames/s",
                              "value": out["tracked_frames_per_s"], "n_gpus": world, "steps": args.steps,
                              "warmup": args.warmup, "batch256": out}), flush=True)
        if world > 1:
            torch.distributed.destroy_process_group()
        return 0
    cal, scene, poses = make_workload(seed, args.frames)
    segs = segments(args.frames)
    frames = [f for _, fr in segs for f in fr]
    plan = step_plan(segs)
    gray, depth = render_frames_gpu(cal, scene, poses, seed, torch)
    stream = torch.cuda.Stream()
    batch = make_batch(cal, len(segs), stream.cuda_stream)
    tile = None
    if args.tile:
        batch.set_icp_chunks_per_cta([int(v) for v in args.tile.split(",")])
        tile = {"icp_chunks_per_cta": batch.icp_chunks_per_cta(), "autotuned": False}
    elif not args.no_tune:
        # tile shape of the linearisation kernel, timed on the first frame of
        # every segment before any timed region (poses do not depend on it)
        from recon_gb300.tune import autotune_icp_chunks
        batch.set_reference([gray[k] for k, _ in segs], [depth[k] for k, _ in segs])
        batch.set_current([gray[fr[0]] for _, fr in segs], [depth[fr[0]] for _, fr in segs])
        chosen, table = autotune_icp_chunks(batch)
        tile = {"icp_chunks_per_cta": chosen[:4],
                "candidates_ms": {str(l): {str(c): round(v, 3) for c, v in t.items()} for l, t in table.items()}}

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()

    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)

    def timed(b, src_g, src_d, out):
        """W warm-up steps, then K steps between a barrier + synchronize on both
        sides; (device ms, wall ms), slowest rank."""
        for _ in range(args.warmup):
            run_step(b, plan, src_g, src_d, out)
        barrier()
        t0 = time.perf_counter()
        e0.record(stream)
        for _ in range(args.steps):
            run_step(b, plan, src_g, src_d, out)
        e1.record(stream)
        barrier()
        wall = time.perf_counter() - t0
        ms = e0.elapsed_time(e1)
        return max_over_ranks(ms, world, "cuda"), max_over_ranks(1000.0 * wall, world, "cuda")

    # -------- plain GPU tracker (the reference's schedule, bit-identical to the FP32 oracle)
    poses_plain = np.zeros((args.frames + 1, 4, 4), np.float32)
    clk = ClockSampler(local)  # samples clocks over every timed region below
    clk.__enter__()
    launches0 = rg.launch_count()
    ms_plain, _ = timed(batch, gray, depth, poses_plain)
    launches_plain = (rg.launch_count() - launches0) / (args.warmup + args.steps)
    plain_value = job_throughput(world, args.frames, args.steps, ms_plain)

    # -------- per-kernel event timing of the same K steps (a separate pass: the
    # events make every launch direct instead of graph-replayed)
    batch.enable_timing(True)
    batch.work(reset=True)
    batch.timing(reset=True)
    for _ in range(args.steps):
        run_step(batch, plan, gray, depth, poses_plain)
    torch.cuda.synchronize()
    timing = batch.timing(reset=True)
    work = batch.work(reset=True).astype(np.float64)
    batch.enable_timing(False)
    it_ms, it_launches = timing["gn_iteration"]
    bytes_iter = float(work[:, 0].sum() * B_PHOTO + work[:, 1].sum() * B_ICP)
    per_launch_bytes = bytes_iter / max(it_launches, 1)
    per_launch_s = it_ms / 1000.0 / max(it_launches, 1)
    achieved = per_launch_bytes / per_launch_s / 1e9 if per_launch_s > 0 else 0.0
    peak, peak_kind = load_peaks()
    traffic = profiled_traffic()

    # -------- the FP64 oracle of the trajectory (rank 0: the judge of every arm's pose error)
    ref64, fp64_s = None, None
    gh = dh = None
    if rank == 0 and not args.no_cpu:
        gh = gray.cpu().numpy()
        dh = depth.cpu().numpy().view(np.uint16)
        ref64, fp64_s = fp64_trajectory(cal, gh, dh, segs)

    def vs_fp64(p):
        if ref64 is None:
            return None, None
        return error_summary(pose_errors(p, ref64, frames))

    gt = np.zeros_like(poses_plain, dtype=np.float64)
    for k, fr in segs:
        for f in fr:
            gt[f] = synth.relative_pose(poses[k], poses[f])
    plain_vs_gt, _ = error_summary(pose_errors(poses_plain, gt, frames))
    plain_vs64, _ = vs_fp64(poses_plain)

    # -------- learned initialisation + shortened schedule
    params, net_info = load_net_params() if not args.plain_only else (None, None)
    learned = None
    settle = None
    net = None
    if params is not None:
        import recon_gb300.initnet as IN
        net = IN.InitNet(max_batch=len(segs), stream=stream.cuda_stream)
        net.set_params(params)
        batch.set_init_net(net, LEARNED_ITERS)
        poses_learned = np.zeros_like(poses_plain)
        launches0 = rg.launch_count()
        ms_learned, _ = timed(batch, gray, depth, poses_learned)
        launches_learned = (rg.launch_count() - launches0) / (args.warmup + args.steps)
        l64, _ = vs_fp64(poses_learned)
        vs_gt, _ = error_summary(pose_errors(poses_learned, gt, frames))
        # share of frames whose start pose came from the network
        batch.set_reference([gray[k] for k, _ in segs], [depth[k] for k, _ in segs])
        acc = []
        for s_ in range(max(len(fr) for _, fr in segs)):
            idx = [fr[min(s_, len(fr) - 1)] for _, fr in segs]
            batch.set_current([gray[i] for i in idx], [depth[i] for i in idx])
            batch.track()
            acc.append(float(batch.init_choice()[0].mean()))
        raw = job_throughput(world, args.frames, args.steps, ms_learned)
        share = l64["within_bound"] if l64 else 1.0
        learned = {"schedule": list(LEARNED_ITERS), "raw_frames_per_s": raw, "within_bound_share": share,
                   "tracked_frames_per_s": raw * share, "ms_per_step": ms_learned / args.steps,
                   "vs_fp64_oracle": l64, "vs_ground_truth": vs_gt, "learned_start_taken": float(np.mean(acc)),
                   "network": net_info, "gpu_launches_per_step": launches_learned,
                   "per_frame_bound_met": bool(l64 and l64["within_bound"] == 1.0)}
        # the plain start pose (the previous frame's) on the same shortened
        # schedule, and on the shortest schedule that keeps it within the rule
        batch.set_init_net(None)
        for key, sched in (("ablation_plain_start_same_schedule", LEARNED_ITERS),
                           ("ablation_plain_start_rule_schedule", PLAIN_START_RULE_ITERS)):
            for i in range(batch.n):
                batch.set_iterations(i, sched)
            poses_short = np.zeros_like(poses_plain)
            ms_short, _ = timed(batch, gray, depth, poses_short)
            s64, _ = vs_fp64(poses_short)
            short_raw = job_throughput(world, args.frames, args.steps, ms_short)
            sshare = s64["within_bound"] if s64 else 1.0
            learned[key] = {"schedule": list(sched), "raw_frames_per_s": short_raw, "within_bound_share": sshare,
                            "tracked_frames_per_s": short_raw * sshare, "vs_fp64_oracle": s64}
        learned["ratio_vs_plain_start_rule_schedule"] = (
            learned["tracked_frames_per_s"] / learned["ablation_plain_start_rule_schedule"]["tracked_frames_per_s"])
        for i in range(batch.n):
            batch.set_iterations(i, ITERS)

        # the settle rule on the reference's schedule: the previous frame's
        # start (every frame within the bound) and the learned start
        def settle_arm(with_net, tol):
            batch.set_init_net(net if with_net else None, ITERS if with_net else None)
            for i in range(batch.n):
                batch.set_settle(i, *tol)
            p_ = np.zeros_like(poses_plain)
            l0 = rg.launch_count()
            batch.work(reset=True)
            ms_, _ = timed(batch, gray, depth, p_)
            nl = (rg.launch_count() - l0) / (args.warmup + args.steps)
            # executed GN iterations per tracked frame (photometric point-iterations / points)
            it_exec = float(batch.work(reset=True)[:, 0].astype(np.float64).sum()) / N_SELECT / (
                len(plan[1]) * batch.n * (args.warmup + args.steps))
            e64, _ = vs_fp64(p_)
            for i in range(batch.n):
                batch.set_settle(i, 0.0, 0.0)
            r_ = job_throughput(world, args.frames, args.steps, ms_)
            sh_ = e64["within_bound"] if e64 else 1.0
            return {"cap_schedule": list(ITERS), "settle_mm": tol[0], "settle_rot": tol[1],
                    "start": "learned" if with_net else "previous frame", "raw_frames_per_s": r_,
                    "within_bound_share": sh_, "tracked_frames_per_s": r_ * sh_, "ms_per_step": ms_ / args.steps,
                    "vs_fp64_oracle": e64, "gpu_launches_per_step": nl, "gn_iterations_per_frame": it_exec,
                    "per_frame_bound_met": bool(e64 and e64["within_bound"] == 1.0)}, p_

        settle, poses_settle = settle_arm(False, SETTLE)
        settle["vs_ground_truth"], _ = error_summary(pose_errors(poses_settle, gt, frames))
        settle["speedup_vs_plain"] = settle["tracked_frames_per_s"] / plain_value
        settle["learned_start"], _ = settle_arm(True, SETTLE)
        # the headline arm again, for the end-to-end measurement
        batch.set_init_net(net, LEARNED_ITERS)

    # headline: frames tracked within the pose-error bound of the FP64 oracle, per second
    if learned is not None:
        value = learned["tracked_frames_per_s"]
        ms_head = learned["ms_per_step"] * args.steps
        head_launches = learned["gpu_launches_per_step"]
    else:
        value, ms_head, head_launches = plain_value * (plain_vs64["within_bound"] if plain_vs64 else 1.0), ms_plain, \
            launches_plain

    # -------- e2e through the C ABI from pinned host memory (the headline arm)
    e2e = None
    if not args.no_e2e:
        g_host = torch.empty(gray.shape, dtype=torch.uint8, pin_memory=True)
        d_host = torch.empty(depth.shape, dtype=torch.int16, pin_memory=True)
        g_host.copy_(gray)
        d_host.copy_(depth)
        g_np = g_host.numpy()
        d_np = d_host.numpy().view(np.uint16)
        out = np.zeros_like(poses_plain)
        ms_dev, ms_wall = timed(batch, g_np, d_np, out)
        ms_e2e = max(ms_dev, ms_wall)
        e64, _ = vs_fp64(out)
        frac = e64["within_bound"] if e64 else 1.0
        n_ref = len(segs)
        n_cur = max(len(fr) for _, fr in segs) * len(segs)
        h2d = (n_ref + n_cur) * W * H * 3
        d2h = max(len(fr) for _, fr in segs) * len(segs) * (64 + 64)
        e2e = {"value": job_throughput(world, args.frames, args.steps, ms_e2e) * frac, "unit": "frames/s",
               "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
               "raw_frames_per_s": job_throughput(world, args.frames, args.steps, ms_e2e), "within_bound_share": frac}
    # -------- mixed precision (config 3: FP16 images and intensities, BF16
    # photometric Jacobians) on the plain arm's schedule: speed and pose error
    # against the FP64 oracle of the same trajectory
    mixed = None
    if not args.no_mixed:
        mb = make_batch(cal, len(segs), stream.cuda_stream, precision=rg.PRECISION_MIXED)
        mb.set_icp_chunks_per_cta(batch.icp_chunks_per_cta())
        poses_mixed = np.zeros_like(poses_plain)
        ms_mixed, _ = timed(mb, gray, depth, poses_mixed)
        m64, _ = vs_fp64(poses_mixed)
        mixed = {"storage": "FP16 current gray pyramid and reference intensities, BF16 photometric Jacobians; "
                            "FP32 arithmetic, exact fixed-point sums, FP64 solve",
                 "frames_per_s": job_throughput(world, args.frames, args.steps, ms_mixed),
                 "vs_fp64_oracle": m64,
                 "vs_fp32_plain": error_summary(pose_errors(poses_mixed, poses_plain, frames))[0]}
        mb.close()

    # -------- the batched workload (256 mixed-resolution instances): a reported
    # measurement beside the headline, with its own roofline
    batched = None
    if not args.no_batch:
        batched = batch_arm(args, torch, world, rank, 5000 + 7919 * rank)
    c1 = config1_arm(args, torch) if rank == 0 and not args.no_cpu else None
    recon_stream = tsdf_arm(args, torch) if rank == 0 and not args.no_tsdf else None
    kinect = kinect_arm(args, torch) if rank == 0 and not args.no_tsdf else None
    clk.__exit__(None, None, None)
    if net is not None:
        batch.set_init_net(None)

    # -------- CPU baseline: the oracle port on whole segments, 1 thread and all
    # threads, and its pose agreement with the GPU
    cpu = None
    oracle_err = None
    if rank == 0 and not args.no_cpu:
        sample_segs = segs[:1]
        threads = os.cpu_count() or 1
        fps_1, _, n1, dt1 = cpu_track(cal, gh, dh, sample_segs, 1)
        fps_cpu, oposes, n, dt = cpu_track(cal, gh, dh, sample_segs, threads)
        cpu = {"value": fps_cpu, "unit": "frames/s", "cores": threads, "kind": "port",
               "value_1_thread": fps_1, "nproc": os.cpu_count(),
               "sample": f"keyframe segment 0: {n} frames tracked on the plain schedule "
                         f"{'/'.join(map(str, ITERS))} with the first {FUSE_FRAMES} fused into the keyframe "
                         f"(the GPU step's work for one segment); {threads} OpenMP threads {dt:.1f} s, "
                         f"1 thread {dt1:.1f} s"}
        d_t, d_r = [], []
        for f, To in oposes.items():
            et, er = synth.pose_error(To.astype(np.float64), poses_plain[f].astype(np.float64))
            d_t.append(et)
            d_r.append(er)
        oracle_err = {"frames": len(d_t), "max_mm": float(max(d_t)), "max_deg": float(max(d_r)),
                      "bit_identical": bool(all(np.array_equal(oposes[f].view(np.uint32),
                                                               poses_plain[f].view(np.uint32)) for f in oposes))}

    if rank == 0:
        clocks = clk.summary()
        line = {
            "metric": METRIC,
            "value": value, "unit": "frames/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms_head / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "fp32", "data": "synthetic (seeded procedural scene ray-cast on the GPU)",
            "config": {"workload": "bi-objective lambda=0.5, 640x480, 4 levels, 8192 photometric points, 300-frame "
                                   "smooth trajectory, keyframe every 10 frames, each keyframe fusing the depth and "
                                   "colour of its 5 nearest tracked frames on the reconstruction stream, 30 keyframe "
                                   "segments batched",
                       "plain_schedule": list(ITERS),
                       "settle_rule": {"mm": SETTLE[0], "rotation_entry": SETTLE[1], "cap": list(ITERS)},
                       "learned_schedule": list(LEARNED_ITERS) if learned is not None else None,
                       "bound": {"mm": BOUND_MM, "deg": BOUND_DEG,
                                 "against": "FP64 oracle run of the same trajectory (same schedule as the plain arm, "
                                            "fusion included, every operation in double)"},
                       "value_is": "learned-init arm: frames within the bound per second (raw frames/s x in-bound "
                                   "share); learned.raw_frames_per_s and learned.vs_fp64_oracle give both parts; "
                                   "settle: the previous frame's start with the settle rule, every frame in bound",
                       "l2": "inputs larger than L2 (301 frames, 277 MB; ~1.2 GB working set)",
                       "parallelism": f"replicas x{world}",
                       "tile": tile or {"icp_chunks_per_cta": batch.icp_chunks_per_cta(), "autotuned": False}},
            "plain": {"frames_per_s": plain_value, "ms_per_step": ms_plain / args.steps,
                      "vs_fp64_oracle": plain_vs64, "vs_ground_truth": plain_vs_gt,
                      "gpu_launches_per_step": launches_plain},
            "settle": settle,
            "learned": learned,
            "speedup_vs_plain": value / plain_value,
            "fp64_oracle": {"frames": len(frames), "seconds": fp64_s} if ref64 is not None else None,
            "e2e": e2e,
            "gpu_launches": int(round(head_launches * args.steps)),
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic, "kernel": "k_iter",
                         "peak_source": peak_kind,
                         "algorithmic_bytes_per_launch": per_launch_bytes,
                         "avg_launch_ms": per_launch_s * 1000.0,
                         "timing": "per-launch CUDA events on the batch stream, separate K-step pass of the plain arm"},
            "cpu_baseline": cpu,
            "clocks": clocks,
            "pose_error_vs_oracle": oracle_err,
            "kernel_ms": {k: v[0] for k, v in timing.items()},
            "kernel_launches": {k: v[1] for k, v in timing.items()},
            "batch256": batched,
            "mixed_precision": mixed,
            "config1": c1,
            "reconstruction": recon_stream,
            "kinect_preprocessing": kinect,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
