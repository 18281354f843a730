"""Seeded synthetic frame pairs for the tests (rendered by the oracle's CPU twin
of the procedural renderer)."""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

import oracle_lib as O
from recon_gb300 import synth


@dataclass
class Pair:
    W: int
    H: int
    L: int
    cal: synth.Calibration
    g0: np.ndarray
    d0: np.ndarray
    g1: np.ndarray
    d1: np.ndarray
    T_gt: np.ndarray  # reference IR -> current IR (float64)


def frame_pair(W: int, H: int, L: int | None = None, seed: int = 7, deg: float = 2.0, mm: float = 20.0,
               noise: float = 0.01, distortion: bool = False) -> Pair:
    if L is None:
        L = 4 if W >= 640 else 3
    cal = synth.make_calibration(W, H, distortion=distortion)
    sc = synth.make_scene(seed)
    Tref = np.eye(4)
    Tcur = Tref @ synth.offset_pose(seed + 1, deg, mm)
    g0, d0 = O.render_pair(sc, synth.camera_struct(cal, "L", Tref), synth.camera_struct(cal, "R", Tref),
                           noise_rel=noise, noise_seed=seed + 2, frame=0)
    g1, d1 = O.render_pair(sc, synth.camera_struct(cal, "L", Tcur), synth.camera_struct(cal, "R", Tcur),
                           noise_rel=noise, noise_seed=seed + 2, frame=1)
    return Pair(W, H, L, cal, g0, d0, g1, d1, synth.relative_pose(Tref, Tcur))


def n_select_for(W: int, H: int) -> int:
    """min(8192, floor(W*H/2/1024)*1024): 8192 at 320x240 and above."""
    return int(min(8192, (W * H // 2 // 1024) * 1024))


@dataclass
class DepthSequence:
    W: int
    H: int
    cal: synth.Calibration
    K: np.ndarray        # normalised 3x3 intrinsics of the depth camera (float32, 9)
    poses: np.ndarray    # n x 4 x 4 camera -> world (float32)
    dist: list           # n distance maps: depth in mm as float32, 0 = invalid
    depth: list          # the same as uint16


def depth_sequence(W: int, H: int, n: int, seed: int = 5, noise: float = 0.005, step_mm: float = 25.0,
                   step_deg: float = 1.5) -> DepthSequence:
    """n depth frames of a seeded scene along a smooth trajectory (the depth
    camera of the rig, no distortion), for the reconstruction stream."""
    cal = synth.make_calibration(W, H)
    sc = synth.make_scene(seed)
    poses = synth.smooth_trajectory(n, seed + 3, max_step_mm=step_mm, max_step_deg=step_deg)
    dist, depth = [], []
    for f in range(n):
        _, d = O.render_pair(sc, synth.camera_struct(cal, "L", poses[f]), synth.camera_struct(cal, "R", poses[f]),
                             noise_rel=noise, noise_seed=seed + 1, frame=f)
        depth.append(d)
        dist.append(d.astype(np.float32))
    K = O.normalized_K(cal.camera_K("L"), W, H)
    return DepthSequence(W, H, cal, K, poses.astype(np.float32), dist, depth)
