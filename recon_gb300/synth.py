"""Seeded synthetic RGB-D inputs: calibration, procedural scene, trajectories.

The reference feeds its tracker from an OpenGL-rendered scene
(utils/src/Renderer.cpp:137-175) and from Kinect captures; neither exists on the
target machines, so every workload here is a seeded procedural scene (textured
room and boxes) ray-cast by ``csrc/scene.h`` on the GPU, with a bit-identical
CPU twin.  This module builds the scene description, the calibration and the
camera trajectories on the host in float64.
"""
from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass

import numpy as np

MAX_BOXES = 16

# Kinect calibration shipped with the reference (bin/data/calib.xml), in the
# width-normalised form calib/calib.cpp stores (K[0] negated, calib.cpp:150,174).
KL_NORM = np.array([-9.2635892e-01, 0.0, 4.9579810e-01,
                    0.0, 9.2545085e-01, 3.8769043e-01,
                    0.0, 0.0, 1.0])
KR_NORM = np.array([-8.3242439e-01, 0.0, 4.9731016e-01,
                    0.0, 8.3136516e-01, 3.6621381e-01,
                    0.0, 0.0, 1.0])
OM_LR = np.array([-4.0133358e-03, -3.1643531e-03, 8.0978370e-03])
T_LR = np.array([-2.5005434e+01, -2.4804501e-02, 1.2691642e+00])
KC_RIGHT = np.array([2.3702838e-01, -4.5079055e-01, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0])


class SceneStruct(ctypes.Structure):
    """Mirror of ``recon_scene`` in csrc/scene.h."""
    _fields_ = [
        ("room_min", ctypes.c_float * 3),
        ("room_max", ctypes.c_float * 3),
        ("n_boxes", ctypes.c_int32),
        ("seed", ctypes.c_uint32),
        ("box_c", (ctypes.c_float * 3) * MAX_BOXES),
        ("box_h", (ctypes.c_float * 3) * MAX_BOXES),
        ("box_R", (ctypes.c_float * 9) * MAX_BOXES),
    ]


class CameraStruct(ctypes.Structure):
    """Mirror of ``recon_camera`` in csrc/scene.h."""
    _fields_ = [
        ("K", ctypes.c_float * 9),
        ("kc", ctypes.c_float * 5),
        ("Rcw", ctypes.c_float * 9),
        ("tcw", ctypes.c_float * 3),
        ("width", ctypes.c_int32),
        ("height", ctypes.c_int32),
    ]


def rodrigues(om: np.ndarray) -> np.ndarray:
    """Rotation matrix of an axis-angle vector (float64)."""
    om = np.asarray(om, dtype=np.float64)
    th = float(np.linalg.norm(om))
    if th < 1e-15:
        return np.eye(3)
    k = om / th
    Kx = np.array([[0, -k[2], k[1]], [k[2], 0, -k[0]], [-k[1], k[0], 0]])
    return np.eye(3) + math.sin(th) * Kx + (1 - math.cos(th)) * (Kx @ Kx)


def log_so3(R: np.ndarray) -> np.ndarray:
    """Axis-angle vector of a rotation; atan2 form, accurate for small angles."""
    w = 0.5 * np.array([R[2, 1] - R[1, 2], R[0, 2] - R[2, 0], R[1, 0] - R[0, 1]])
    s = float(np.linalg.norm(w))
    c = (np.trace(R) - 1.0) * 0.5
    th = math.atan2(s, c)
    if s < 1e-300:
        return np.zeros(3)
    return w * (th / s)


def se3(R: np.ndarray, t: np.ndarray) -> np.ndarray:
    T = np.eye(4)
    T[:3, :3] = R
    T[:3, 3] = t
    return T


def inv_se3(T: np.ndarray) -> np.ndarray:
    Ti = np.eye(4)
    Ti[:3, :3] = T[:3, :3].T
    Ti[:3, 3] = -T[:3, :3].T @ T[:3, 3]
    return Ti


def pose_error(Ta: np.ndarray, Tb: np.ndarray) -> tuple[float, float]:
    """(translation mm, rotation deg) of Ta^-1 Tb."""
    D = inv_se3(np.asarray(Ta, np.float64)) @ np.asarray(Tb, np.float64)
    return float(np.linalg.norm(D[:3, 3])), float(np.degrees(np.linalg.norm(log_so3(D[:3, :3]))))


@dataclass
class Calibration:
    """Raw (double) calibration plus the 96-float calibData buffer (calib/calib.h:22-37)."""
    width: int
    height: int
    KL: np.ndarray
    KR: np.ndarray
    TLR: np.ndarray
    kcR: np.ndarray
    min_dist: float
    max_dist: float
    calib: np.ndarray  # float32[96]

    @property
    def TRL(self) -> np.ndarray:
        return inv_se3(self.TLR)

    def camera_K(self, which: str) -> np.ndarray:
        src = self.KL if which == "L" else self.KR
        K = np.eye(3, dtype=np.float32)
        K.flat[:6] = (self.width * src[:6]).astype(np.float32)
        return K


def calib_setup(KL: np.ndarray, KR: np.ndarray, TLR: np.ndarray, kc: np.ndarray,
                min_dist: float, max_dist: float, width: int, B: float = 1.7034511, b: float = 75.0) -> np.ndarray:
    """Fill the 96-float calibData buffer (calib/calib.cpp:74-93; c0/c1 from calib.cpp:699-701)."""
    c = np.zeros(96, dtype=np.float32)

    def put_K(off, K):
        M = np.eye(3, dtype=np.float32).reshape(-1)
        M[:6] = (width * np.asarray(K[:6], np.float64)).astype(np.float32)
        c[off:off + 9] = M
        det = np.linalg.det(M.astype(np.float64).reshape(3, 3))
        inv = np.eye(3) if abs(det) < 1e-5 else np.linalg.inv(M.astype(np.float64).reshape(3, 3))
        c[off + 9:off + 18] = inv.reshape(-1).astype(np.float32)

    put_K(0, KR)
    c[18:26] = np.asarray(kc, np.float64)[:8].astype(np.float32)
    c[26:42] = np.asarray(TLR, np.float64).reshape(-1).astype(np.float32)
    c[64:80] = inv_se3(np.asarray(TLR, np.float64)).reshape(-1).astype(np.float32)
    put_K(43, KL)
    scale = 1.0 / (8 * b * abs(KL[0]) * 640.0)
    c[42] = np.float32(-scale)
    c[61] = np.float32(B * 640.0 * scale)
    c[62] = np.float32(min_dist)
    c[63] = np.float32(max_dist)
    return c


def make_calibration(width: int, height: int, distortion: bool = False,
                     min_dist: float = 400.0, max_dist: float = 4500.0) -> Calibration:
    """calibData for a width x height image, following calib/calib.cpp:74-93.

    The reference scales every intrinsic row by the image width (calib.cpp:78,84).
    """
    R = rodrigues(OM_LR)
    TLR = se3(R, T_LR)
    kc = KC_RIGHT.copy() if distortion else np.zeros(8)
    calib = calib_setup(KL_NORM, KR_NORM, TLR, kc, min_dist, max_dist, width)
    return Calibration(width, height, KL_NORM.copy(), KR_NORM.copy(), TLR, kc, min_dist, max_dist, calib)


def make_scene(seed: int, n_boxes: int = 7) -> SceneStruct:
    """Seeded room (5 m x 3 m x 4.8 m) with textured walls and n_boxes boxes.

    The camera starts at the origin looking down -z; visible depths fall in
    roughly 500-4000 mm.
    """
    rng = np.random.default_rng(seed)
    sc = SceneStruct()
    sc.room_min[:] = [-2600.0, -1300.0, -4000.0]
    sc.room_max[:] = [2600.0, 1600.0, 800.0]
    sc.seed = np.uint32(seed * 2654435761 % (1 << 32))
    n_boxes = min(n_boxes, MAX_BOXES)
    sc.n_boxes = n_boxes
    for b in range(n_boxes):
        depth = rng.uniform(900.0, 3200.0)
        x = rng.uniform(-0.45, 0.45) * depth
        h = rng.uniform([150.0, 150.0, 150.0], [550.0, 500.0, 450.0])
        on_floor = rng.random() < 0.6
        y = (-1300.0 + h[1]) if on_floor else rng.uniform(-0.3, 0.3) * depth
        yaw = rng.uniform(-0.6, 0.6)
        pitch = rng.uniform(-0.25, 0.25) if not on_floor else 0.0
        Rw = rodrigues(np.array([pitch, yaw, 0.0]))
        sc.box_c[b][:] = [x, y, -depth]
        sc.box_h[b][:] = h.tolist()
        sc.box_R[b][:] = Rw.T.reshape(-1).astype(np.float32).tolist()  # world -> local
    return sc


def camera_struct(calib: Calibration, which: str, T_wc: np.ndarray) -> CameraStruct:
    """Camera for the IR ('L', depth) or RGB ('R', gray) view.

    T_wc is the IR camera-to-world pose; the RGB camera is T_wc * TRL
    (TLR maps IR coordinates to RGB coordinates, calib.cpp:655-675).
    """
    cam = CameraStruct()
    cam.K[:] = calib.camera_K(which).reshape(-1).tolist()
    if which == "R":
        cam.kc[:] = [float(np.float32(calib.kcR[i])) for i in range(5)]
        T = T_wc @ calib.TRL
    else:
        cam.kc[:] = [0.0] * 5
        T = T_wc
    cam.Rcw[:] = T[:3, :3].astype(np.float32).reshape(-1).tolist()
    cam.tcw[:] = T[:3, 3].astype(np.float32).tolist()
    cam.width = calib.width
    cam.height = calib.height
    return cam


def smooth_trajectory(n_frames: int, seed: int, max_step_mm: float = 12.0, max_step_deg: float = 0.8) -> np.ndarray:
    """Camera-to-world IR poses [n_frames, 4, 4] (float64) of a smooth random motion.

    Sums of sinusoids with per-frame speed bounded by max_step_mm / max_step_deg
    (below the 5 cm / 3 degree per-frame bound of the bi-objective workload).
    """
    rng = np.random.default_rng(seed)
    t = np.arange(n_frames, dtype=np.float64)
    pos = np.zeros((n_frames, 3))
    rot = np.zeros((n_frames, 3))
    for axis in range(3):
        for _ in range(3):
            f = rng.uniform(1.0 / 160.0, 1.0 / 45.0)
            ph = rng.uniform(0, 2 * math.pi)
            amp = max_step_mm / (2 * math.pi * f) / 3.0 / math.sqrt(3.0)
            pos[:, axis] += amp * np.sin(2 * math.pi * f * t + ph)
            fr = rng.uniform(1.0 / 160.0, 1.0 / 45.0)
            phr = rng.uniform(0, 2 * math.pi)
            ampr = math.radians(max_step_deg) / (2 * math.pi * fr) / 3.0 / math.sqrt(3.0)
            rot[:, axis] += ampr * np.sin(2 * math.pi * fr * t + phr)
    pos -= pos[0]
    rot -= rot[0]
    poses = np.zeros((n_frames, 4, 4))
    for i in range(n_frames):
        poses[i] = se3(rodrigues(rot[i]), pos[i])
    return poses


def offset_pose(seed: int, deg: float, mm: float) -> np.ndarray:
    """Rigid offset: rotation of `deg` about a random axis and `mm` along a random direction."""
    rng = np.random.default_rng(seed)
    ax = rng.normal(size=3)
    ax /= np.linalg.norm(ax)
    tr = rng.normal(size=3)
    tr /= np.linalg.norm(tr)
    return se3(rodrigues(ax * math.radians(deg)), tr * mm)


def relative_pose(T_w_ref: np.ndarray, T_w_cur: np.ndarray) -> np.ndarray:
    """Ground-truth tracker pose: reference IR coordinates -> current IR coordinates."""
    return inv_se3(T_w_cur) @ T_w_ref
