"""ctypes binding of the CPU oracle (oracle/liboracle.so).

Test infrastructure: imported only by the tests, smoke() and bench.py's CPU
baseline leg.  Builds the oracle with its Makefile on first use.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")
LIB_PATH = os.path.join(ORACLE_DIR, "liboracle.so")

GEOMETRIC, PHOTOMETRIC, BIOBJECTIVE = 0, 1, 2
CHOLESKY, CG = 0, 1

_lock = threading.Lock()
_lib = None


class OrcConfig(ctypes.Structure):
    _fields_ = [
        ("width", ctypes.c_int32), ("height", ctypes.c_int32), ("levels", ctypes.c_int32),
        ("n_select", ctypes.c_int32), ("hist_bins", ctypes.c_int32), ("select_bins", ctypes.c_int32),
        ("solver", ctypes.c_int32), ("mode", ctypes.c_int32), ("lambda_", ctypes.c_float),
        ("iters", ctypes.c_int32 * 4), ("opt_scale_in", ctypes.c_float), ("opt_scale_out", ctypes.c_float),
        ("precision", ctypes.c_int32), ("settle_mm", ctypes.c_float), ("settle_rot", ctypes.c_float),
    ]


class OrcIterTrace(ctypes.Structure):
    _fields_ = [
        ("level", ctypes.c_int32), ("iter", ctypes.c_int32), ("mode", ctypes.c_int32),
        ("solved", ctypes.c_int32), ("icp_selected", ctypes.c_int32), ("status", ctypes.c_int32),
        ("T", ctypes.c_float * 16),
        ("A", ctypes.c_double * 36), ("b", ctypes.c_double * 6),
        ("A_ph", ctypes.c_double * 36), ("b_ph", ctypes.c_double * 6),
        ("A_icp", ctypes.c_double * 36), ("b_icp", ctypes.c_double * 6),
        ("hist", ctypes.c_int32 * 256), ("median_bin", ctypes.c_int32), ("pad_", ctypes.c_int32),
    ]


class OrcTsdfParams(ctypes.Structure):
    _fields_ = [("R", ctypes.c_int32), ("origin", ctypes.c_float * 3), ("dim", ctypes.c_float * 3),
                ("W", ctypes.c_int32), ("H", ctypes.c_int32), ("min_dist", ctypes.c_float),
                ("max_dist", ctypes.c_float)]


def _build() -> None:
    src = [os.path.join(ORACLE_DIR, f) for f in ("oracle.c", "oracle_fp64.c", "oracle.h", "initnet_oracle.c",
                                                 "Makefile")]
    src.append(os.path.join(ROOT, "recon_gb300", "csrc", "scene.h"))
    if os.path.exists(LIB_PATH) and all(os.path.getmtime(LIB_PATH) >= os.path.getmtime(s) for s in src):
        return
    subprocess.run(["make", "-s", "-C", ORACLE_DIR], check=True)


def lib() -> ctypes.CDLL:
    global _lib
    with _lock:
        if _lib is None:
            _build()
            L = ctypes.CDLL(LIB_PATH)
            vp = ctypes.c_void_p
            i32 = ctypes.c_int
            f32 = ctypes.c_float
            L.orc_create.restype = vp
            L.orc_create.argtypes = [ctypes.POINTER(OrcConfig), vp]
            L.orc_destroy.argtypes = [vp]
            L.orc_set_reference.argtypes = [vp, vp, vp]
            L.orc_set_reference_float.argtypes = [vp, vp, vp]
            L.orc_set_current.argtypes = [vp, vp, vp]
            L.orc_track.argtypes = [vp, vp, vp, i32]
            L.orc_get_array.argtypes = [vp, ctypes.c_char_p, i32, vp, ctypes.c_int64]
            L.orc_n_icp_selected.argtypes = [vp, i32]
            L.orc_render_depth.argtypes = [vp, vp, f32, ctypes.c_uint32, ctypes.c_uint32, vp]
            L.orc_render_gray.argtypes = [vp, vp, vp]
            L.orc_expm_update.argtypes = [vp, vp, ctypes.c_double]
            L.orc_expm_twist.argtypes = [vp, vp]
            L.orc_solve_cholesky.argtypes = [vp, vp, vp]
            L.orc_solve_cg.argtypes = [vp, vp, ctypes.c_double, i32, vp]
            L.orc_reduce27.argtypes = [vp, vp, i32, vp, vp]
            L.orc_f16_round.argtypes = [f32]
            L.orc_f16_round.restype = f32
            L.orc_bf16_round.argtypes = [f32]
            L.orc_bf16_round.restype = f32
            L.orc_reduce27_refordered.argtypes = [vp, vp, i32, vp, vp]
            L.orc_fx_add.argtypes = [vp, f32, vp]
            L.orc_fx_to_double.argtypes = [vp]
            L.orc_fx_to_double.restype = ctypes.c_double
            L.orc_fx27_clear.argtypes = [vp]
            L.orc_reduce27_fx.argtypes = [vp, vp, i32, vp]
            L.orc_fx27_value.argtypes = [vp, vp, vp]
            L.orc_net_param_count.restype = ctypes.c_int64
            L.orc_net_coarse.argtypes = [vp, vp, i32, i32, i32, vp]
            L.orc_net_forward.argtypes = [vp, vp, i32, i32, vp]
            L.orc_net_loss_grad.argtypes = [vp, vp, vp, i32, i32, vp]
            L.orc_net_loss_grad.restype = ctypes.c_double
            L.orc_generate_weights.argtypes = [vp, vp, i32, i32, vp, vp, vp]
            L.orc_student_t.argtypes = [vp, i32, vp]
            L.orc_filter_indices.argtypes = [vp, i32, vp, i32, i32, vp]
            L.orc_grad_histogram.argtypes = [vp, i32, i32, vp]
            L.orc_fuse_depth.argtypes = [vp, i32, i32, vp, i32, vp, vp, f32, vp, vp]
            L.orc_zmap_to_xyz.argtypes = [vp, i32, i32, vp, vp]
            L.orc_zmap_to_xyz6.argtypes = [vp, i32, i32, vp, vp, vp]
            L.orc_xyz2cloud.argtypes = [vp, i32, i32, vp, vp, vp]
            L.orc_add_vertex_attributes.argtypes = [vp, i32, vp, i32, i32, vp, vp, i32]
            L.orc_precompute_jacobian.argtypes = [vp, i32, vp, vp, f32, i32, vp]
            L.orc_interpolate_residual.argtypes = [i32, vp, vp, vp, vp, i32, vp, i32, i32, vp, i32, i32, vp, vp]
            L.orc_downsample2.argtypes = [vp, i32, i32, vp]
            L.orc_gen_cloud6.argtypes = [vp, i32, i32, vp, vp, vp]
            L.orc_compute_normals6.argtypes = [vp, vp, i32, i32]
            L.orc_downsample_cloud6.argtypes = [vp, vp, i32, i32, vp, vp]
            L.orc_icp_residual_mask.argtypes = [vp, vp, i32, i32, vp, vp, vp, vp, i32, vp, vp]
            L.orc_icp_residual_jacobian.argtypes = [vp, vp, i32, i32, i32, i32, vp, vp, vp, vp, i32, vp, vp, vp, f32]
            L.orc_icp_residual_jacobian_grid.argtypes = [vp, i32, i32, i32, vp, vp, vp, vp, i32, vp, vp, vp, f32]
            L.orc_compact.argtypes = [vp, i32, vp]
            L.orc_compact.restype = i32
            L.orc_generate_weights.restype = i32
            L.orc_filter_indices.restype = i32
            L.orc_solve_cholesky.restype = i32
            L.orc_linear_fuse.argtypes = [vp, vp, ctypes.c_double, i32, vp, vp, ctypes.c_double, i32]
            L.orc_convert_gray.argtypes = [vp, i32, vp]
            L.orc_convert_depth.argtypes = [vp, i32, vp]
            L.orc_rgbd_float4_to_gray_z.argtypes = [vp, i32, i32, vp, vp, vp]
            L.orc_fuse_keyframe.argtypes = [vp, i32, vp, vp, f32]
            L.orc_fuse_keyframe_rgbd.argtypes = [vp, i32, vp, vp, vp, f32]
            L.orc64_create.restype = vp
            L.orc64_create.argtypes = [ctypes.POINTER(OrcConfig), vp]
            L.orc64_destroy.argtypes = [vp]
            L.orc64_set_reference.argtypes = [vp, vp, vp]
            L.orc64_set_current.argtypes = [vp, vp, vp]
            L.orc64_fuse_keyframe.argtypes = [vp, i32, vp, vp, vp, ctypes.c_double]
            L.orc64_track.argtypes = [vp, vp]
            L.orc64_get_pose.argtypes = [vp, vp]
            L.orc64_set_pose.argtypes = [vp, vp]
            L.orc64_get_array.argtypes = [vp, ctypes.c_char_p, i32, vp, ctypes.c_int64]
            L.orc_fuse_rgbd.argtypes = [vp, vp, i32, i32, vp, i32, vp, vp, vp, f32, vp, vp, vp]
            L.orc_xyz2cloud_col.argtypes = [vp, i32, i32, vp, vp, vp, vp]
            L.orc_init_gate.argtypes = [vp, vp, vp]
            L.orc_init_gate.restype = i32
            L.orc_set_pose.argtypes = [vp, vp]
            L.orc_get_pose.argtypes = [vp, vp]
            L.orc_kinect_d2z.argtypes = [vp, i32, i32, f32, f32, f32, f32, f32, f32, vp]
            L.orc_kinect_d2z_low.argtypes = [vp, i32, i32, f32, f32, f32, f32, f32, f32, vp]
            L.orc_kinect_rgb2gray.argtypes = [vp, i32, i32, vp]
            L.orc_kinect_undistort.argtypes = [vp, i32, i32, vp, vp, vp, vp]
            L.orc_kinect_disparity_to_float.argtypes = [vp, i32, vp]
            L.orc_kinect_depth_normalized.argtypes = [vp, vp, i32, i32, f32, f32, f32, f32, f32, f32, vp]
            L.orc_kinect_rgb_to_hdr.argtypes = [vp, i32, vp]
            L.orc_kinect_rgb_to_gray_hdr.argtypes = [vp, i32, vp]
            L.orc_kinect_rgb_hdr_to_gray.argtypes = [vp, i32, vp]
            L.orc_kinect_undistort_rgb_hdr.argtypes = [vp, i32, i32, vp, vp, vp, vp]
            L.orc_gen_oriented_points6.argtypes = [vp, vp, i32, i32, vp, vp]
            L.orc_set_reference_oriented.argtypes = [vp, vp, vp, vp, vp]
            L.orc_tsdf_invert_rt4.argtypes = [vp, vp]
            L.orc_tsdf_reset.argtypes = [vp, ctypes.c_int64]
            L.orc_tsdf_dist_from_rgbd.argtypes = [vp, i32, i32, f32, f32, vp]
            L.orc_tsdf_update.argtypes = [vp, ctypes.POINTER(OrcTsdfParams), vp, vp, vp]
            L.orc_tsdf_raycast.argtypes = [vp, ctypes.POINTER(OrcTsdfParams), vp, vp, i32, vp]
            L.orc_tsdf_shade.argtypes = [vp, i32, i32, vp, vp]
            L.orc_tsdf_resample.argtypes = [vp, vp, ctypes.POINTER(OrcTsdfParams), vp]
            L.orc_pose_settled.argtypes = [vp, vp, f32, f32]
            L.orc_pose_settled.restype = i32
            L.orc_num_threads.restype = i32
            L.orc_set_threads.argtypes = [i32]
            _lib = L
    return _lib


def ptr(a: np.ndarray) -> ctypes.c_void_p:
    """Address of a numpy array.  The caller must keep `a` referenced until the
    call that uses the address returns (bind temporaries to a name first)."""
    assert a.flags["C_CONTIGUOUS"]
    return ctypes.c_void_p(a.ctypes.data)


def ptrs(arrays) -> ctypes.Array:
    """C array of pointers (const float *const *) to the given numpy arrays."""
    arr = (ctypes.c_void_p * len(arrays))()
    for i, a in enumerate(arrays):
        assert a.flags["C_CONTIGUOUS"]
        arr[i] = a.ctypes.data
    return arr


def make_config(width, height, levels, mode=PHOTOMETRIC, iters=(1, 3, 10, 5), n_select=8192, hist_bins=64,
                select_bins=256, solver=CHOLESKY, lam=0.5, precision=0, settle=(0.0, 0.0)) -> OrcConfig:
    c = OrcConfig()
    c.width, c.height, c.levels = width, height, levels
    c.n_select, c.hist_bins, c.select_bins = n_select, hist_bins, select_bins
    c.solver, c.mode, c.lambda_ = solver, mode, lam
    it = list(iters) + [0] * (4 - len(iters))
    c.iters[:] = it[:4]
    c.opt_scale_in, c.opt_scale_out = 1e-3, 1e3
    c.precision = precision
    c.settle_mm, c.settle_rot = settle
    return c


class OracleTracker:
    """Operator-level oracle tracker (PhotoTracker + ShapeTracker schedule)."""

    def __init__(self, cfg: OrcConfig, calib: np.ndarray):
        self.L = lib()
        self.cfg = cfg
        self.calib = np.ascontiguousarray(calib, dtype=np.float32)
        self.h = self.L.orc_create(ctypes.byref(cfg), ptr(self.calib))

    def close(self):
        if self.h:
            self.L.orc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_reference(self, gray: np.ndarray, depth: np.ndarray):
        g = np.ascontiguousarray(gray, np.uint8)
        d = np.ascontiguousarray(depth, np.uint16)
        self.L.orc_set_reference(self.h, ptr(g), ptr(d))

    def set_reference_oriented(self, gray, depth, points, normals):
        """The filtered reference: ICP level 0 from float4 point and normal maps."""
        g = np.ascontiguousarray(gray, np.uint8)
        d = np.ascontiguousarray(depth, np.uint16)
        p = np.ascontiguousarray(points, np.float32).reshape(-1)
        n = np.ascontiguousarray(normals, np.float32).reshape(-1)
        self.L.orc_set_reference_oriented(self.h, ptr(g), ptr(d), ptr(p), ptr(n))

    def set_reference_float(self, gray: np.ndarray, z: np.ndarray):
        """A reference given as float gray in [0, 1] and z = -mm (0 or NaN: invalid)."""
        g = np.ascontiguousarray(gray, np.float32).reshape(-1)
        zz = np.ascontiguousarray(z, np.float32).reshape(-1)
        self.L.orc_set_reference_float(self.h, ptr(g), ptr(zz))

    def set_current(self, gray: np.ndarray, depth: np.ndarray):
        g = np.ascontiguousarray(gray, np.uint8)
        d = np.ascontiguousarray(depth, np.uint16)
        self.L.orc_set_current(self.h, ptr(g), ptr(d))

    def track(self, T: np.ndarray | None = None, max_trace: int = 64):
        Tin = np.eye(4, dtype=np.float32) if T is None else np.ascontiguousarray(T, np.float32).copy()
        trace = (OrcIterTrace * max_trace)()
        n = self.L.orc_track(self.h, ptr(Tin), ctypes.cast(trace, ctypes.c_void_p), max_trace)
        if n < 0:
            raise RuntimeError("oracle track failed")
        return Tin.reshape(4, 4), list(trace)[:min(n, max_trace)]

    def pose(self) -> np.ndarray:
        T = np.zeros(16, np.float32)
        self.L.orc_get_pose(self.h, ptr(T))
        return T.reshape(4, 4)

    def init_gate(self, net_out: np.ndarray, scale: np.ndarray) -> int:
        """The learned start-pose gate (orc_init_gate) with the network output of the GPU."""
        y = np.ascontiguousarray(net_out, np.float32)
        sc = np.ascontiguousarray(scale, np.float32)
        return int(self.L.orc_init_gate(self.h, ptr(y), ptr(sc)))

    def fuse_keyframe(self, depths, Ts, gate: float = 30.0, grays=None):
        """Keyframe fusion of depth (and, with grays, colour) of tracked frames."""
        ds = [np.ascontiguousarray(d, np.uint16) for d in depths]
        T = np.ascontiguousarray(np.asarray(Ts, np.float32).reshape(len(ds), 16))
        if grays is None:
            rc = self.L.orc_fuse_keyframe(self.h, len(ds), ptrs(ds), ptr(T), gate)
        else:
            gs = [np.ascontiguousarray(g, np.uint8) for g in grays]
            rc = self.L.orc_fuse_keyframe_rgbd(self.h, len(ds), ptrs(gs), ptrs(ds), ptr(T), gate)
        if rc != 0:
            raise RuntimeError("oracle fuse failed")

    def get(self, name: str, level: int, shape, dtype) -> np.ndarray:
        out = np.zeros(shape, dtype=dtype)
        n = self.L.orc_get_array(self.h, name.encode(), level, ptr(out), out.nbytes)
        if n < 0:
            raise KeyError(name)
        return out.reshape(-1)[: n // out.itemsize].reshape(-1)


class Oracle64Tracker:
    """The FP64 oracle (orc64_*): the same tracker with every operation in
    double and the pose kept in double; the judge of pose error."""

    def __init__(self, cfg: OrcConfig, calib: np.ndarray):
        self.L = lib()
        self._calib = np.ascontiguousarray(calib, np.float32).reshape(96)
        self.h = self.L.orc64_create(ctypes.byref(cfg), ptr(self._calib))
        self.W, self.H, self.P = cfg.width, cfg.height, cfg.n_select

    def close(self):
        if self.h:
            self.L.orc64_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_reference(self, gray, depth):
        g = np.ascontiguousarray(gray, np.uint8)
        d = np.ascontiguousarray(depth, np.uint16)
        self.L.orc64_set_reference(self.h, ptr(g), ptr(d))

    def set_current(self, gray, depth):
        g = np.ascontiguousarray(gray, np.uint8)
        d = np.ascontiguousarray(depth, np.uint16)
        self.L.orc64_set_current(self.h, ptr(g), ptr(d))

    def track(self, T=None) -> np.ndarray:
        """The plain schedule from T (None: the tracker's pose); the FP64 pose."""
        Tio = np.empty(16, np.float64)
        if T is None:
            self.L.orc64_get_pose(self.h, ptr(Tio))
        else:
            Tio[:] = np.asarray(T, np.float64).reshape(16)
        if self.L.orc64_track(self.h, ptr(Tio)) < 0:
            raise RuntimeError("oracle64 track failed")
        return Tio.reshape(4, 4)

    def fuse_keyframe(self, depths, Ts, gate: float = 30.0, grays=None):
        ds = [np.ascontiguousarray(d, np.uint16) for d in depths]
        T = np.ascontiguousarray(np.asarray(Ts, np.float64).reshape(len(ds), 16))
        gs = None if grays is None else [np.ascontiguousarray(g, np.uint8) for g in grays]
        gp = None if gs is None else ptrs(gs)
        if self.L.orc64_fuse_keyframe(self.h, len(ds), gp, ptrs(ds), ptr(T), gate) != 0:
            raise RuntimeError("oracle64 fuse failed")

    def get(self, name: str, level: int, count: int, dtype) -> np.ndarray:
        out = np.zeros(count, dtype=dtype)
        n = self.L.orc64_get_array(self.h, name.encode(), level, ptr(out), out.nbytes)
        if n < 0:
            raise KeyError(name)
        return out[: n // out.itemsize]


def render_pair(scene, cam_ir, cam_rgb, noise_rel=0.01, noise_seed=1, frame=0):
    L = lib()
    d = np.zeros((cam_ir.height, cam_ir.width), np.uint16)
    g = np.zeros((cam_rgb.height, cam_rgb.width), np.uint8)
    L.orc_render_depth(ctypes.byref(scene), ctypes.byref(cam_ir), noise_rel, noise_seed, frame, ptr(d))
    L.orc_render_gray(ctypes.byref(scene), ctypes.byref(cam_rgb), ptr(g))
    return g, d


# ---- reconstruction stream (oracle_tsdf.c) ----
# the reference's grid placement (VoxelGrid.cpp:62-65: kinect8 test)
TSDF_ORIGIN = (0.0, 0.01, -1600.01)
TSDF_DIM = (1500.0, 1500.0, 1500.0)


def tsdf_params(R, W, H, min_dist=400.0, max_dist=4500.0, origin=TSDF_ORIGIN, dim=TSDF_DIM) -> OrcTsdfParams:
    p = OrcTsdfParams()
    p.R, p.W, p.H = R, W, H
    p.origin[:] = list(origin)
    p.dim[:] = list(dim)
    p.min_dist, p.max_dist = min_dist, max_dist
    return p


def normalized_K(K_pix, W, H) -> np.ndarray:
    """getNormalizedK (main.cpp:878-882): pixel intrinsics over width / height, in float."""
    K = np.asarray(K_pix, np.float32).reshape(-1)
    out = np.zeros(9, np.float32)
    out[0] = K[0] / np.float32(W)
    out[2] = K[2] / np.float32(W)
    out[4] = K[4] / np.float32(H)
    out[5] = K[5] / np.float32(H)
    out[8] = 1.0
    return out


class OracleTSDF:
    """The CPU oracle's voxel grid: reset, update, ray cast, shading, resampling."""

    def __init__(self, params: OrcTsdfParams):
        self.p = params
        self.grid = np.zeros(2 * params.R ** 3, np.float32)
        lib().orc_tsdf_reset(ptr(self.grid), params.R ** 3)

    def update(self, dist, Tcur, K):
        d = np.ascontiguousarray(dist, np.float32).reshape(-1)
        T = np.ascontiguousarray(Tcur, np.float32).reshape(-1)
        Kn = np.ascontiguousarray(K, np.float32).reshape(-1)
        lib().orc_tsdf_update(ptr(self.grid), ctypes.byref(self.p), ptr(d), ptr(T), ptr(Kn))

    def raycast(self, Tcur, K, filtering=True):
        xyz = np.zeros(4 * self.p.W * self.p.H, np.float32)
        T = np.ascontiguousarray(Tcur, np.float32).reshape(-1)
        Kn = np.ascontiguousarray(K, np.float32).reshape(-1)
        lib().orc_tsdf_raycast(ptr(self.grid), ctypes.byref(self.p), ptr(T), ptr(Kn), int(filtering), ptr(xyz))
        return xyz

    def shade(self, xyz):
        shaded = np.zeros_like(xyz)
        normal = np.zeros_like(xyz)
        lib().orc_tsdf_shade(ptr(xyz), self.p.W, self.p.H, ptr(shaded), ptr(normal))
        return shaded, normal

    def resampled(self, Tcur):
        dst = np.zeros_like(self.grid)
        T = np.ascontiguousarray(Tcur, np.float32).reshape(-1)
        lib().orc_tsdf_resample(ptr(dst), ptr(self.grid), ctypes.byref(self.p), ptr(T))
        return dst
