"""recon_gb300: GB300-native dense RGB-D tracking (the hot path of ttykkala/recon).

The compute path is librecon_track.so (hand-written sm_103a CUDA behind the C
ABI of include/recon_track.h).  This module is a thin ctypes layer over that
ABI mirroring the reference's operator classes (PhotoTracker / ShapeTracker,
tracker/tracker/phototracker.h:33-154): set a reference, set a current frame,
track.  There is no CPU fallback: when the CUDA library cannot be loaded every
call raises.
"""
from __future__ import annotations

import ctypes
import os
import threading

import numpy as np

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG_DIR, "librecon_track.so")

GEOMETRIC, PHOTOMETRIC, BIOBJECTIVE = 0, 1, 2
# status codes (include/recon_track.h)
OK, ERR_INVALID_ARG, ERR_NOT_ENOUGH_POINTS, ERR_NON_SPD, ERR_TIMEOUT, ERR_CUDA, ERR_STATE, ERR_NO_DEVICE = \
    0, -1, -2, -3, -4, -5, -6, -7
SOLVER_CHOLESKY, SOLVER_CG = 0, 1
PRECISION_FP32, PRECISION_MIXED = 0, 1
CALIB_SIZE = 96

RECON_OK = 0
ERRORS = {
    -1: "invalid argument", -2: "not enough points", -3: "non-SPD normal equations",
    -4: "timeout", -5: "CUDA error", -6: "reference or current frame missing", -7: "no CUDA device",
}


class ReconError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class Config(ctypes.Structure):
    """recon_config (include/recon_track.h)."""
    _fields_ = [
        ("width", ctypes.c_int32), ("height", ctypes.c_int32), ("levels", ctypes.c_int32),
        ("n_select", ctypes.c_int32), ("hist_bins", ctypes.c_int32), ("select_bins", ctypes.c_int32),
        ("solver", ctypes.c_int32), ("mode", ctypes.c_int32), ("lambda_", ctypes.c_float),
        ("iters", ctypes.c_int32 * 4), ("opt_scale_in", ctypes.c_float), ("opt_scale_out", ctypes.c_float),
        ("precision", ctypes.c_int32), ("settle_mm", ctypes.c_float), ("settle_rot", ctypes.c_float),
        ("reserved", ctypes.c_int32 * 5),
    ]


class TrackStats(ctypes.Structure):
    _fields_ = [
        ("status", ctypes.c_int32), ("iterations", ctypes.c_int32), ("solves", ctypes.c_int32),
        ("icp_selected", ctypes.c_int32 * 4), ("photo_median_bin", ctypes.c_int32), ("non_spd", ctypes.c_int32),
        ("reserved", ctypes.c_int32 * 5),
    ]


class IterTrace(ctypes.Structure):
    _fields_ = [
        ("level", ctypes.c_int32), ("iter", ctypes.c_int32), ("mode", ctypes.c_int32),
        ("solved", ctypes.c_int32), ("icp_selected", ctypes.c_int32), ("status", ctypes.c_int32),
        ("T", ctypes.c_float * 16),
        ("A", ctypes.c_double * 36), ("b", ctypes.c_double * 6),
        ("A_ph", ctypes.c_double * 36), ("b_ph", ctypes.c_double * 6),
        ("A_icp", ctypes.c_double * 36), ("b_icp", ctypes.c_double * 6),
        ("hist", ctypes.c_int32 * 256), ("median_bin", ctypes.c_int32), ("pad_", ctypes.c_int32),
    ]


def make_config(width: int, height: int, levels: int | None = None, mode: int = PHOTOMETRIC,
                iters=(1, 3, 10, 5), n_select: int = 8192, hist_bins: int = 64, select_bins: int = 256,
                solver: int = SOLVER_CHOLESKY, lam: float = 0.5, precision: int = PRECISION_FP32,
                settle=(0.0, 0.0)) -> Config:
    """Tracker configuration; defaults follow phototracker.cpp (8192 points,
    iterations {1,3,10,5} coarse->fine, 3 levels at 320 wide and 4 at 640).
    `settle` = (mm, rotation entry) tolerances of the early level exit
    (recon_batch_set_settle); (0, 0) keeps the reference's fixed schedule."""
    if levels is None:
        levels = 4 if width >= 640 else 3
    c = Config()
    c.width, c.height, c.levels = width, height, levels
    c.n_select, c.hist_bins, c.select_bins = n_select, hist_bins, select_bins
    c.solver, c.mode, c.lambda_ = solver, mode, lam
    it = list(iters)[:levels] + [0] * (4 - min(len(iters), levels))
    c.iters[:] = it[:4]
    c.opt_scale_in, c.opt_scale_out = 1e-3, 1e3
    c.precision = precision
    c.settle_mm, c.settle_rot = settle
    return c


_lock = threading.Lock()
_lib = None


def lib() -> ctypes.CDLL:
    """Loads librecon_track.so (built by recon_gb300.build / __graft_entry__.build)."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise ImportError(f"{LIB_PATH} is missing: build it with `python -m recon_gb300.build` "
                                  "(there is no CPU fallback)")
            L = ctypes.CDLL(LIB_PATH)
            vp, i32, i64, f32 = ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64, ctypes.c_float
            L.recon_last_error.restype = ctypes.c_char_p
            L.recon_batch_create.argtypes = [i32, vp, vp, vp, ctypes.POINTER(vp)]
            L.recon_batch_destroy.argtypes = [vp]
            L.recon_batch_size.argtypes = [vp]
            L.recon_batch_set_reference.argtypes = [vp, vp, vp, i32]
            L.recon_batch_set_reference_rgbd_float4.argtypes = [vp, i32, vp, i32]
            L.recon_batch_set_reference_oriented.argtypes = [vp, vp, vp, vp, vp, i32]
            L.recon_set_reference_oriented.argtypes = [vp, vp, vp, vp, vp, i32]
            L.recon_batch_set_current.argtypes = [vp, vp, vp, i32]
            L.recon_batch_set_current_rgbd_float4.argtypes = [vp, i32, vp, i32]
            L.recon_batch_track.argtypes = [vp, vp, vp]
            L.recon_batch_track_async.argtypes = [vp, vp]
            L.recon_batch_get_poses.argtypes = [vp, vp, vp]
            L.recon_batch_set_iterations.argtypes = [vp, i32, vp]
            L.recon_batch_set_settle.argtypes = [vp, i32, ctypes.c_float, ctypes.c_float]
            L.recon_set_settle.argtypes = [vp, ctypes.c_float, ctypes.c_float]
            L.recon_batch_set_mode.argtypes = [vp, i32, i32, f32]
            L.recon_batch_set_icp_chunks_per_cta.argtypes = [vp, vp]
            L.recon_batch_get_icp_chunks_per_cta.argtypes = [vp, vp]
            L.recon_batch_enable_trace.argtypes = [vp, i32]
            L.recon_batch_get_trace.argtypes = [vp, i32, vp, i32]
            L.recon_batch_get_array.argtypes = [vp, i32, ctypes.c_char_p, i32, vp, i64]
            L.recon_batch_set_init_net.argtypes = [vp, vp, vp]
            L.recon_batch_get_init.argtypes = [vp, vp, vp]
            L.recon_batch_get_array.restype = i64
            L.recon_calib_setup.argtypes = [vp, vp, vp, vp, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                            ctypes.c_double, i32, vp]
            L.recon_tracker_create.argtypes = [vp, vp, vp, ctypes.POINTER(vp)]
            L.recon_tracker_destroy.argtypes = [vp]
            L.recon_set_reference.argtypes = [vp, vp, vp, i32]
            L.recon_set_current.argtypes = [vp, vp, vp, i32]
            L.recon_track.argtypes = [vp, vp, vp]
            L.recon_set_iterations.argtypes = [vp, vp]
            L.recon_set_mode.argtypes = [vp, i32, f32]
            L.recon_get_relative_pose.argtypes = [vp, vp]
            L.recon_get_global_pose.argtypes = [vp, vp]
            L.recon_pose_difference_exceeded.argtypes = [vp, f32, f32]
            L.recon_set_reference_updating.argtypes = [vp, i32, f32, f32]
            L.recon_reference_outdated.argtypes = [vp]
            L.recon_batch_reference_outdated.argtypes = [vp, f32, f32, vp]
            L.recon_reset.argtypes = [vp]
            L.recon_batch_track_sequence.argtypes = [vp, i32, vp, vp, i32, vp, vp]
            L.recon_batch_fuse_keyframe.argtypes = [vp, i32, vp, vp, i32, f32]
            L.recon_batch_fuse_keyframe_rgbd.argtypes = [vp, i32, vp, vp, vp, i32, f32]
            L.recon_batch_fuse_sequence.argtypes = [vp, i32, f32]
            L.recon_batch_enable_timing.argtypes = [vp, i32]
            L.recon_batch_get_timing.argtypes = [vp, vp, vp, i32]
            L.recon_batch_get_work.argtypes = [vp, vp, i32]
            L.recon_batch_stream.argtypes = [vp]
            L.recon_batch_stream.restype = vp
            L.recon_launch_count.restype = i64
            L.recon_render_depth.argtypes = [vp, vp, f32, ctypes.c_uint32, ctypes.c_uint32, vp, vp]
            L.recon_render_gray.argtypes = [vp, vp, vp, vp]
            L.recon_selftest_exact_arith.argtypes = [vp]
            L.recon_kinect_disparity_to_depth.argtypes = [vp, i32, i32, f32, f32, f32, f32, f32, f32, i32, vp, vp]
            L.recon_kinect_rgb_to_gray.argtypes = [vp, i32, i32, vp, vp]
            L.recon_kinect_undistort_gray.argtypes = [vp, i32, i32, vp, vp, vp, vp, vp]
            L.recon_kinect_disparity_to_float.argtypes = [vp, i32, i32, vp, vp]
            L.recon_kinect_depth_normalized.argtypes = [vp, vp, i32, i32, f32, f32, f32, f32, f32, f32, vp, vp]
            L.recon_kinect_rgb_to_hdr.argtypes = [vp, i32, i32, vp, vp]
            L.recon_kinect_rgb_to_gray_hdr.argtypes = [vp, vp, i32, i32, vp, vp]
            L.recon_kinect_undistort_rgb_hdr.argtypes = [vp, i32, i32, vp, vp, vp, vp, vp]
            L.recon_trajectory_save.argtypes = [ctypes.c_char_p, vp, i32, i32, i32]
            L.recon_trajectory_load.argtypes = [ctypes.c_char_p, vp, i32, i32]
            L.recon_trajectory_load.restype = i32
            L.recon_track_params_load.argtypes = [ctypes.c_char_p, vp, vp, vp, i32]
            L.recon_track_params_load.restype = i32
            L.recon_track_params_lookup.argtypes = [vp, i32, i32]
            L.recon_track_params_lookup.restype = i32
            L.recon_tsdf_default_params.argtypes = [i32, i32, i32, f32, f32, ctypes.POINTER(TsdfParams)]
            L.recon_tsdf_default_params.restype = None
            L.recon_tsdf_create.argtypes = [ctypes.POINTER(TsdfParams), vp, ctypes.POINTER(vp)]
            L.recon_tsdf_destroy.argtypes = [vp]
            L.recon_tsdf_reset.argtypes = [vp]
            L.recon_tsdf_set_dist_map.argtypes = [vp, vp, i32]
            L.recon_tsdf_set_dist_rgbd_float4.argtypes = [vp, vp, i32]
            L.recon_tsdf_set_dist_depth16.argtypes = [vp, vp, i32]
            L.recon_tsdf_update.argtypes = [vp, vp, vp]
            L.recon_tsdf_raycast.argtypes = [vp, vp, vp, i32]
            L.recon_tsdf_resample.argtypes = [vp, vp, vp]
            L.recon_tsdf_device_array.argtypes = [vp, ctypes.c_char_p]
            L.recon_tsdf_device_array.restype = vp
            L.recon_tsdf_get.argtypes = [vp, ctypes.c_char_p, vp, i64]
            L.recon_tsdf_get.restype = i64
            L.recon_tsdf_set_grid.argtypes = [vp, vp, i32]
            L.recon_tsdf_stream.argtypes = [vp]
            L.recon_tsdf_stream.restype = vp
            L.recon_tsdf_enable_timing.argtypes = [vp, i32]
            L.recon_tsdf_get_timing.argtypes = [vp, vp, vp, i32]
            L.recon_tsdf_enable_counting.argtypes = [vp, i32]
            L.recon_tsdf_get_counts.argtypes = [vp, vp, i32]
            _lib = L
    return _lib


class TsdfParams(ctypes.Structure):
    """recon_tsdf_params (include/recon_tsdf.h)."""
    _fields_ = [("grid_resolution", ctypes.c_int32), ("cube_origin", ctypes.c_float * 3),
                ("cube_dim", ctypes.c_float * 3), ("width", ctypes.c_int32), ("height", ctypes.c_int32),
                ("min_dist", ctypes.c_float), ("max_dist", ctypes.c_float)]


def check(rc: int) -> int:
    if rc < 0:
        raise ReconError(rc, lib().recon_last_error().decode())
    return rc


def _ptr(a) -> ctypes.c_void_p:
    """Address of a C-contiguous numpy array or a torch tensor."""
    if isinstance(a, np.ndarray):
        assert a.flags["C_CONTIGUOUS"]
        return ctypes.c_void_p(a.ctypes.data)
    if hasattr(a, "data_ptr"):
        assert a.is_contiguous()
        return ctypes.c_void_p(a.data_ptr())
    raise TypeError(type(a))


def _on_device(a) -> int:
    return int(hasattr(a, "is_cuda") and a.is_cuda)


def _order_after_torch(batch) -> None:
    """The batch reads device inputs on its own stream: make that stream wait
    for the work already queued on torch's current stream (which may still be
    writing the tensors being passed).  An event and a wait, no host stall."""
    import torch
    torch.cuda.ExternalStream(batch.stream()).wait_stream(torch.cuda.current_stream())


class DeviceView:
    """A device array owned by the library (no copy): the address, shape and
    the stream that writes it, with enough of the tensor interface for these
    wrappers (and __cuda_array_interface__ for torch.as_tensor)."""

    is_cuda = True

    def __init__(self, ptr: int, shape, typestr: str, stream: int, owner):
        self.ptr, self.shape, self.typestr, self.stream, self.owner = ptr, tuple(shape), typestr, stream, owner

    def data_ptr(self) -> int:
        return self.ptr

    def is_contiguous(self) -> bool:
        return True

    @property
    def __cuda_array_interface__(self):
        return {"shape": self.shape, "typestr": self.typestr, "data": (self.ptr, False), "version": 3,
                "stream": None}


def _after_producer(consumer, a) -> None:
    """Orders the consumer's stream after the work that produces `a`: the
    owning library stream of a DeviceView, else torch's current stream."""
    if isinstance(a, DeviceView):
        import torch
        torch.cuda.ExternalStream(consumer.stream()).wait_stream(torch.cuda.ExternalStream(a.stream))
    elif _on_device(a):
        _order_after_torch(consumer)


class Batch:
    """Several tracker instances served by the same launches (recon_batch_*)."""

    def __init__(self, configs, calibs, stream=None):
        L = lib()
        self.n = len(configs)
        self.configs = list(configs)
        self._resolutions = {(c.width, c.height) for c in self.configs}
        cfg_arr = (Config * self.n)(*configs)
        cal = np.ascontiguousarray(np.stack([np.asarray(c, np.float32).reshape(CALIB_SIZE) for c in calibs]))
        self._calib = cal
        h = ctypes.c_void_p()
        st = ctypes.c_void_p(stream) if stream else None
        check(L.recon_batch_create(self.n, ctypes.cast(cfg_arr, ctypes.c_void_p), _ptr(cal), st, ctypes.byref(h)))
        self.h = h
        self._keep = []

    def close(self):
        if getattr(self, "h", None):
            lib().recon_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _ptr_tables(self, grays, depths):
        g = (ctypes.c_void_p * self.n)()
        d = (ctypes.c_void_p * self.n)()
        dev = None
        keep = []
        for i in range(self.n):
            if grays[i] is None:
                continue
            gi, di = grays[i], depths[i]
            if isinstance(gi, np.ndarray):
                gi = np.ascontiguousarray(gi, np.uint8)
                di = np.ascontiguousarray(di, np.uint16)
            keep += [gi, di]
            od = _on_device(gi)
            if dev is None:
                dev = od
            elif dev != od:
                raise ValueError("mix of host and device inputs")
            g[i] = _ptr(gi).value
            d[i] = _ptr(di).value
        if dev:
            _order_after_torch(self)
        return g, d, int(dev or 0), keep

    def _stack_table(self, stack, index, itemsize):
        """Addresses of frames `index` (an integer array of any shape) of a
        C-contiguous frame stack [F, H, W] (numpy array or torch tensor, host
        or CUDA) as a uint64 pointer table, computed with numpy: base + index
        times the frame's bytes.  Every instance must have the stack's
        resolution.  Returns (table, on_device)."""
        if isinstance(stack, np.ndarray):
            if not stack.flags["C_CONTIGUOUS"]:
                raise ValueError("frame stack must be C-contiguous")
            base, dev, esz = stack.ctypes.data, 0, stack.itemsize
        elif hasattr(stack, "data_ptr"):
            if not stack.is_contiguous():
                raise ValueError("frame stack must be contiguous")
            base, dev, esz = stack.data_ptr(), int(stack.is_cuda), stack.element_size()
        else:
            raise TypeError(type(stack))
        if len(stack.shape) != 3 or esz != itemsize:
            raise ValueError(f"frame stack must be [frames, H, W] of {itemsize}-byte elements")
        F, H, W = (int(v) for v in stack.shape)
        if self._resolutions != {(W, H)}:
            raise ValueError(f"instance resolutions {sorted(self._resolutions)} differ from the stack's {W}x{H}")
        idx = np.asarray(index, np.int64)
        if idx.size and (idx.min() < 0 or idx.max() >= F):
            raise IndexError("frame index out of the stack")
        table = np.uint64(base) + idx.astype(np.uint64) * np.uint64(H * W * itemsize)
        if dev:
            _order_after_torch(self)
        return np.ascontiguousarray(table, np.uint64), dev

    def _stack_tables(self, grays, depths, index, shape):
        idx = np.asarray(index, np.int64)
        if idx.shape != shape:
            raise ValueError(f"frame index must have shape {shape}")
        g, dg = self._stack_table(grays, idx, 1)
        d, dd = self._stack_table(depths, idx, 2)
        if dg != dd:
            raise ValueError("mix of host and device inputs")
        return g, d, dg

    def set_reference_frames(self, grays, depths, index):
        """set_reference from frame stacks: instance i takes frame index[i] of
        grays [F, H, W] uint8 and depths [F, H, W] uint16 (or int16)."""
        g, d, dev = self._stack_tables(grays, depths, index, (self.n,))
        check(lib().recon_batch_set_reference(self.h, g.ctypes.data, d.ctypes.data, dev))

    def set_current_frames(self, grays, depths, index):
        """set_current from frame stacks (as set_reference_frames)."""
        g, d, dev = self._stack_tables(grays, depths, index, (self.n,))
        self._keep = [grays, depths]
        check(lib().recon_batch_set_current(self.h, g.ctypes.data, d.ctypes.data, dev))

    def track_sequence_frames(self, grays, depths, index):
        """track_sequence from frame stacks: frame f of instance i is
        index[f, i] of grays [F, H, W] uint8 and depths [F, H, W] uint16 (or
        int16).  Returns poses [nf, n, 4, 4] and the last frame's stats."""
        idx = np.asarray(index, np.int64)
        if idx.ndim != 2:
            raise ValueError("frame index must be [frames, instances]")
        nf = idx.shape[0]
        g, d, dev = self._stack_tables(grays, depths, idx, (nf, self.n))
        T = np.zeros((nf, self.n, 16), np.float32)
        stats = (TrackStats * self.n)()
        check(lib().recon_batch_track_sequence(self.h, nf, g.ctypes.data, d.ctypes.data, dev, _ptr(T),
                                               ctypes.cast(stats, ctypes.c_void_p)))
        return T.reshape(nf, self.n, 4, 4), list(stats)

    def set_reference(self, grays, depths):
        g, d, dev, keep = self._ptr_tables(grays, depths)
        check(lib().recon_batch_set_reference(self.h, ctypes.cast(g, ctypes.c_void_p),
                                              ctypes.cast(d, ctypes.c_void_p), dev))

    def set_current(self, grays, depths):
        g, d, dev, keep = self._ptr_tables(grays, depths)
        self._keep = keep
        check(lib().recon_batch_set_current(self.h, ctypes.cast(g, ctypes.c_void_p),
                                            ctypes.cast(d, ctypes.c_void_p), dev))

    def set_reference_oriented(self, grays, depths, points, normals):
        """The filtered reference (recon_batch_set_reference_oriented): ICP
        level 0 of instance i from the float4 maps points[i] / normals[i]
        (e.g. TSDF.view("xyz") / TSDF.view("normal")), None for the raw path."""
        g, d, dev, keep = self._ptr_tables(grays, depths)
        p = (ctypes.c_void_p * self.n)()
        q = (ctypes.c_void_p * self.n)()
        for i in range(self.n):
            if points[i] is None or normals[i] is None:
                continue
            pi, ni = points[i], normals[i]
            if isinstance(pi, np.ndarray):
                pi = np.ascontiguousarray(pi, np.float32)
                ni = np.ascontiguousarray(ni, np.float32)
            if _on_device(pi) != bool(dev) or _on_device(ni) != bool(dev):
                raise ValueError("mix of host and device inputs")
            _after_producer(self, pi)
            _after_producer(self, ni)
            keep += [pi, ni]
            p[i] = _ptr(pi).value
            q[i] = _ptr(ni).value
        check(lib().recon_batch_set_reference_oriented(self.h, ctypes.cast(g, ctypes.c_void_p),
                                                       ctypes.cast(d, ctypes.c_void_p), ctypes.cast(p, ctypes.c_void_p),
                                                       ctypes.cast(q, ctypes.c_void_p), dev))

    def set_reference_rgbd_float4(self, inst: int, rgbd):
        a = np.ascontiguousarray(rgbd, np.float32) if isinstance(rgbd, np.ndarray) else rgbd
        if _on_device(a):
            _order_after_torch(self)
        check(lib().recon_batch_set_reference_rgbd_float4(self.h, inst, _ptr(a), _on_device(a)))

    def set_current_rgbd_float4(self, inst: int, rgbd):
        a = np.ascontiguousarray(rgbd, np.float32) if isinstance(rgbd, np.ndarray) else rgbd
        if _on_device(a):
            _order_after_torch(self)
        check(lib().recon_batch_set_current_rgbd_float4(self.h, inst, _ptr(a), _on_device(a)))

    def track(self, T_init=None):
        """Returns (poses [n,4,4] float32, stats list)."""
        T = np.zeros((self.n, 16), np.float32)
        if T_init is not None:
            T[:] = np.asarray(T_init, np.float32).reshape(self.n, 16)
        stats = (TrackStats * self.n)()
        if T_init is None:
            check(lib().recon_batch_track_async(self.h, None))
            check(lib().recon_batch_get_poses(self.h, _ptr(T), ctypes.cast(stats, ctypes.c_void_p)))
        else:
            check(lib().recon_batch_track(self.h, _ptr(T), ctypes.cast(stats, ctypes.c_void_p)))
        return T.reshape(self.n, 4, 4), list(stats)

    def track_sequence(self, grays, depths):
        """grays/depths: nf lists of n images (host arrays or CUDA tensors).
        Returns poses [nf, n, 4, 4] and the last frame's stats."""
        nf = len(grays)
        g = (ctypes.c_void_p * (nf * self.n))()
        d = (ctypes.c_void_p * (nf * self.n))()
        dev = None
        keep = []
        for f in range(nf):
            for i in range(self.n):
                gi, di = grays[f][i], depths[f][i]
                if isinstance(gi, np.ndarray):
                    gi = np.ascontiguousarray(gi, np.uint8)
                    di = np.ascontiguousarray(di, np.uint16)
                keep += [gi, di]
                od = _on_device(gi)
                if dev is None:
                    dev = od
                elif dev != od:
                    raise ValueError("mix of host and device inputs")
                g[f * self.n + i] = _ptr(gi).value
                d[f * self.n + i] = _ptr(di).value
        if dev:
            _order_after_torch(self)
        T = np.zeros((nf, self.n, 16), np.float32)
        stats = (TrackStats * self.n)()
        check(lib().recon_batch_track_sequence(self.h, nf, ctypes.cast(g, ctypes.c_void_p),
                                               ctypes.cast(d, ctypes.c_void_p), int(dev or 0), _ptr(T),
                                               ctypes.cast(stats, ctypes.c_void_p)))
        return T.reshape(nf, self.n, 4, 4), list(stats)

    def fuse_keyframe(self, depths, T, gate_mm: float = 30.0, grays=None):
        """Keyframe fusion (recon_batch_fuse_keyframe_rgbd).  depths (and
        optionally grays): nframes lists of n images; T: [nframes, n, 4, 4]
        keyframe -> frame poses."""
        nf = len(depths)
        d = (ctypes.c_void_p * (nf * self.n))()
        g = (ctypes.c_void_p * (nf * self.n))() if grays is not None else None
        dev = None
        keep = []
        for f in range(nf):
            for i in range(self.n):
                di = depths[f][i]
                if isinstance(di, np.ndarray):
                    di = np.ascontiguousarray(di, np.uint16)
                keep.append(di)
                od = _on_device(di)
                dev = od if dev is None else dev
                d[f * self.n + i] = _ptr(di).value
                if g is not None:
                    gi = grays[f][i]
                    if isinstance(gi, np.ndarray):
                        gi = np.ascontiguousarray(gi, np.uint8)
                    keep.append(gi)
                    if _on_device(gi) != od:
                        raise ValueError("mix of host and device inputs")
                    g[f * self.n + i] = _ptr(gi).value
        if dev:
            _order_after_torch(self)
        Tn = np.ascontiguousarray(np.asarray(T, np.float32).reshape(nf * self.n, 16))
        check(lib().recon_batch_fuse_keyframe_rgbd(self.h, nf, None if g is None else ctypes.cast(g, ctypes.c_void_p),
                                                   ctypes.cast(d, ctypes.c_void_p), _ptr(Tn), int(dev or 0), gate_mm))

    def fuse_sequence(self, nframes: int, gate_mm: float = 30.0):
        """Fuses the first nframes frames of the last tracked sequence (depth
        and colour, tracked poses) into the keyframes, all on the device
        (recon_batch_fuse_sequence)."""
        check(lib().recon_batch_fuse_sequence(self.h, int(nframes), float(gate_mm)))

    def track_async(self, T_init=None):
        T = None if T_init is None else np.ascontiguousarray(np.asarray(T_init, np.float32).reshape(self.n, 16))
        check(lib().recon_batch_track_async(self.h, None if T is None else _ptr(T)))

    def poses(self):
        T = np.zeros((self.n, 16), np.float32)
        stats = (TrackStats * self.n)()
        check(lib().recon_batch_get_poses(self.h, _ptr(T), ctypes.cast(stats, ctypes.c_void_p)))
        return T.reshape(self.n, 4, 4), list(stats)

    def set_iterations(self, inst: int, iters):
        it = (ctypes.c_int32 * 4)(*(list(iters) + [0] * 4)[:4])
        check(lib().recon_batch_set_iterations(self.h, inst, ctypes.cast(it, ctypes.c_void_p)))

    def set_mode(self, inst: int, mode: int, lam: float):
        check(lib().recon_batch_set_mode(self.h, inst, mode, lam))

    def set_settle(self, inst: int, tol_mm: float, tol_rot: float):
        """Early level exit of an instance once its pose has settled (0, 0: off)."""
        check(lib().recon_batch_set_settle(self.h, inst, tol_mm, tol_rot))

    def set_icp_chunks_per_cta(self, per_level):
        """ICP chunks of 1024 pixels per linearisation CTA at each level (0: built-in)."""
        v = (ctypes.c_int32 * 4)(*(list(per_level) + [0] * 4)[:4])
        check(lib().recon_batch_set_icp_chunks_per_cta(self.h, ctypes.cast(v, ctypes.c_void_p)))

    def icp_chunks_per_cta(self):
        v = (ctypes.c_int32 * 4)()
        check(lib().recon_batch_get_icp_chunks_per_cta(self.h, ctypes.cast(v, ctypes.c_void_p)))
        return list(v)

    def enable_trace(self, max_iters: int):
        check(lib().recon_batch_enable_trace(self.h, max_iters))

    def trace(self, inst: int, max_iters: int = 256):
        buf = (IterTrace * max_iters)()
        n = check(lib().recon_batch_get_trace(self.h, inst, ctypes.cast(buf, ctypes.c_void_p), max_iters))
        return list(buf)[:n]

    def set_init_net(self, net, iters=None):
        """Attaches a learned initialisation network (recon_gb300.initnet.InitNet)
        with schedule `iters` (coarse to fine); None detaches it."""
        if net is None:
            check(lib().recon_batch_set_init_net(self.h, None, None))
            self._net = None
            return
        it = (ctypes.c_int32 * 4)(*(list(iters) + [0] * 4)[:4])
        check(lib().recon_batch_set_init_net(self.h, net.h, ctypes.cast(it, ctypes.c_void_p)))
        self._net = net  # keep it alive while attached

    def init_choice(self):
        """The last frame's learned start-pose decisions [n] and network outputs [n, 6]."""
        ch = np.zeros(self.n, np.int32)
        out = np.zeros((self.n, 6), np.float32)
        check(lib().recon_batch_get_init(self.h, _ptr(ch), _ptr(out)))
        return ch, out

    def get_array(self, inst: int, name: str, level: int, dtype, count: int) -> np.ndarray:
        out = np.zeros(count, dtype)
        n = check(lib().recon_batch_get_array(self.h, inst, name.encode(), level, _ptr(out), out.nbytes))
        return out[: n // out.itemsize]


TIMING_KINDS = ["gn_iteration", "icp_mask", "icp_student_t", "prep_current", "prep_reference", "gn_solve",
                "icp_prepare", "keyframe_fusion"]


def launch_count() -> int:
    return int(lib().recon_launch_count())


def selftest_exact_arith() -> int:
    """Mismatches of the Student-t passes' truncation against the conversion
    over every float in [0, 2^23), run on the current GPU."""
    out = np.zeros(1, np.int64)
    check(lib().recon_selftest_exact_arith(out.ctypes.data))
    return int(out[0])


def _batch_extras():
    def enable_timing(self, on: bool = True):
        check(lib().recon_batch_enable_timing(self.h, int(on)))

    def timing(self, reset: bool = False):
        ms = np.zeros(8, np.float64)
        cnt = np.zeros(8, np.int64)
        k = check(lib().recon_batch_get_timing(self.h, _ptr(ms), _ptr(cnt), int(reset)))
        return {TIMING_KINDS[i]: (float(ms[i]), int(cnt[i])) for i in range(k)}

    def work(self, reset: bool = False) -> np.ndarray:
        out = np.zeros((self.n, 4), np.uint64)
        check(lib().recon_batch_get_work(self.h, _ptr(out), int(reset)))
        return out

    def stream(self) -> int:
        return int(lib().recon_batch_stream(self.h) or 0)

    Batch.enable_timing = enable_timing
    Batch.timing = timing
    Batch.work = work
    Batch.stream = stream


_batch_extras()


class Tracker(Batch):
    """PhotoTracker-style single tracker (recon_tracker_* = batch of one)."""

    def __init__(self, config: Config, calib, stream=None):
        super().__init__([config], [calib], stream)

    def _frame(self, gray, depth):
        if isinstance(gray, np.ndarray):
            gray = np.ascontiguousarray(gray, np.uint8)
            depth = np.ascontiguousarray(depth, np.uint16)
        if _on_device(gray) != _on_device(depth):
            raise ValueError("mix of host and device inputs")
        if _on_device(gray):
            _order_after_torch(self)
        return gray, depth, _on_device(gray)

    def set_reference(self, gray, depth):
        """recon_set_reference: the new keyframe; the relative pose restarts at the identity."""
        g, d, dev = self._frame(gray, depth)
        check(lib().recon_set_reference(self.h, _ptr(g), _ptr(d), dev))

    def set_reference_oriented(self, gray, depth, points, normals):
        """recon_set_reference_oriented: the filtered reference (ICP points and
        normals from float4 maps, e.g. a TSDF ray cast); the relative pose
        restarts at the identity."""
        g, d, dev = self._frame(gray, depth)
        if isinstance(points, np.ndarray):
            points = np.ascontiguousarray(points, np.float32)
            normals = np.ascontiguousarray(normals, np.float32)
        if _on_device(points) != bool(dev) or _on_device(normals) != bool(dev):
            raise ValueError("mix of host and device inputs")
        _after_producer(self, points)
        _after_producer(self, normals)
        check(lib().recon_set_reference_oriented(self.h, _ptr(g), _ptr(d), _ptr(points), _ptr(normals), dev))

    def set_current(self, gray, depth):
        g, d, dev = self._frame(gray, depth)
        self._keep = [g, d]
        check(lib().recon_set_current(self.h, _ptr(g), _ptr(d), dev))

    def track(self, T_init=None):
        """recon_track: the schedule from T_init (None: the tracker's pose) and
        the host pose bookkeeping (applyIncrement).  Returns the tracked pose
        (reference -> current) and the frame's statistics; a frame whose status
        is RECON_ERR_NON_SPD or RECON_ERR_NOT_ENOUGH_POINTS keeps its pose and
        is reported in the statistics, not raised."""
        stats = (TrackStats * 1)()
        T = None
        if T_init is not None:
            # a copy: recon_track writes the result into its pose argument
            T = np.array(T_init, dtype=np.float32).reshape(16).copy()
        rc = lib().recon_track(self.h, None if T is None else _ptr(T), ctypes.cast(stats, ctypes.c_void_p))
        if rc < 0 and rc not in (ERR_NON_SPD, ERR_NOT_ENOUGH_POINTS):
            check(rc)
        if T is None:
            T = np.zeros(16, np.float32)
            check(lib().recon_batch_get_poses(self.h, _ptr(T), None))
        return T.reshape(4, 4), stats[0]

    def global_pose(self) -> np.ndarray:
        g = np.zeros(16, np.float64)
        check(lib().recon_get_global_pose(self.h, _ptr(g)))
        return g.reshape(4, 4)

    def relative_pose(self) -> np.ndarray:
        """The host relative pose (current -> reference, float), getRelativePose."""
        T = np.zeros(16, np.float32)
        check(lib().recon_get_relative_pose(self.h, _ptr(T)))
        return T.reshape(4, 4)

    def set_reference_updating(self, on: bool, dist_mm: float = 125.0, angle_deg: float = 12.5):
        check(lib().recon_set_reference_updating(self.h, int(on), dist_mm, angle_deg))

    def reference_outdated(self) -> bool:
        return bool(check(lib().recon_reference_outdated(self.h)))

    def reset(self):
        check(lib().recon_reset(self.h))


def pose_difference_exceeded(dT, dist_mm: float = 125.0, angle_deg: float = 12.5) -> bool:
    """poseDifferenceExceeded (recon_pose_difference_exceeded): host code, no GPU needed."""
    T = np.ascontiguousarray(np.asarray(dT, np.float32).reshape(16))
    return bool(check(lib().recon_pose_difference_exceeded(_ptr(T), dist_mm, angle_deg)))


def _batch_reference_outdated(self, dist_mm: float = 125.0, angle_deg: float = 12.5) -> np.ndarray:
    out = np.zeros(self.n, np.int32)
    check(lib().recon_batch_reference_outdated(self.h, dist_mm, angle_deg, _ptr(out)))
    return out.astype(bool)


Batch.reference_outdated = _batch_reference_outdated


def render_depth(scene, camera, noise_rel: float, noise_seed: int, frame: int, out, stream=None):
    """Ray-casts uint16 depth (mm) into the device tensor `out` (recon_render_depth)."""
    check(lib().recon_render_depth(ctypes.byref(scene), ctypes.byref(camera), noise_rel, noise_seed, frame,
                                   _ptr(out), ctypes.c_void_p(stream) if stream else None))


def render_gray(scene, camera, out, stream=None):
    check(lib().recon_render_gray(ctypes.byref(scene), ctypes.byref(camera), _ptr(out),
                                  ctypes.c_void_p(stream) if stream else None))


# ---- reconstruction stream (include/recon_tsdf.h) ----

TSDF_TIMING_KINDS = ("update", "raycast", "shading", "distance_map", "reset_resample")


def tsdf_params(grid_resolution: int, width: int, height: int, min_dist: float = 400.0, max_dist: float = 4500.0,
                cube_origin=None, cube_dim=None) -> TsdfParams:
    """VoxelGrid's parameters; the reference's grid placement unless given."""
    p = TsdfParams()
    lib().recon_tsdf_default_params(grid_resolution, width, height, min_dist, max_dist, ctypes.byref(p))
    if cube_origin is not None:
        p.cube_origin[:] = [float(v) for v in cube_origin]
    if cube_dim is not None:
        p.cube_dim[:] = [float(v) for v in cube_dim]
    return p


def normalized_K(K_pix, width: int, height: int) -> np.ndarray:
    """getNormalizedK (main.cpp:878-882): pixel intrinsics over width / height, in float."""
    K = np.asarray(K_pix, np.float32).reshape(-1)
    out = np.zeros(9, np.float32)
    out[0] = K[0] / np.float32(width)
    out[2] = K[2] / np.float32(width)
    out[4] = K[4] / np.float32(height)
    out[5] = K[5] / np.float32(height)
    out[8] = 1.0
    return out


class TSDF:
    """A voxel grid of the reconstruction stream (VoxelGrid, recon_tsdf_*).

    Poses are 4x4 camera -> world; K is the normalised 3x3 intrinsic matrix.
    Device inputs (torch tensors) are read on the grid's stream after the work
    queued on torch's current stream."""

    def __init__(self, params: TsdfParams, stream=None):
        self.params = params
        h = ctypes.c_void_p()
        check(lib().recon_tsdf_create(ctypes.byref(params), ctypes.c_void_p(stream) if stream else None,
                                      ctypes.byref(h)))
        self.h = h
        self.R = params.grid_resolution
        self.W, self.H = params.width, params.height

    def close(self):
        if getattr(self, "h", None):
            lib().recon_tsdf_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def stream(self) -> int:
        return lib().recon_tsdf_stream(self.h)

    def _inputs_ready(self, a):
        if _on_device(a):
            _order_after_torch(self)

    def reset(self):
        check(lib().recon_tsdf_reset(self.h))

    def set_dist_map(self, dist):
        self._inputs_ready(dist)
        check(lib().recon_tsdf_set_dist_map(self.h, _ptr(dist), _on_device(dist)))

    def set_dist_rgbd_float4(self, rgbd):
        self._inputs_ready(rgbd)
        check(lib().recon_tsdf_set_dist_rgbd_float4(self.h, _ptr(rgbd), _on_device(rgbd)))

    def set_dist_depth16(self, depth):
        self._inputs_ready(depth)
        check(lib().recon_tsdf_set_dist_depth16(self.h, _ptr(depth), _on_device(depth)))

    @staticmethod
    def _f32(a, n):
        a = np.ascontiguousarray(np.asarray(a, np.float32).reshape(-1))
        assert a.size == n
        return a

    def update(self, T, K):
        T = self._f32(T, 16)
        K = self._f32(K, 9)
        check(lib().recon_tsdf_update(self.h, _ptr(T), _ptr(K)))

    def raycast(self, T, K, cubic_filter: bool = True):
        T = self._f32(T, 16)
        K = self._f32(K, 9)
        check(lib().recon_tsdf_raycast(self.h, _ptr(T), _ptr(K), int(cubic_filter)))

    def resample_from(self, src: "TSDF", T):
        T = self._f32(T, 16)
        check(lib().recon_tsdf_resample(self.h, src.h, _ptr(T)))

    def device_array(self, name: str) -> int:
        p = lib().recon_tsdf_device_array(self.h, name.encode())
        if not p:
            raise ReconError(ERR_INVALID_ARG, f"unknown array {name}")
        return p

    def view(self, name: str) -> DeviceView:
        """A no-copy view of a device array ("xyz", "normal", "shaded": H x W x 4
        float; "dist": H x W float; "tsdf": R x R x R x 2 float)."""
        shape = {"xyz": (self.H, self.W, 4), "normal": (self.H, self.W, 4), "shaded": (self.H, self.W, 4),
                 "dist": (self.H, self.W), "tsdf": (self.R, self.R, self.R, 2)}[name]
        return DeviceView(self.device_array(name), shape, "<f4", self.stream(), self)

    def get(self, name: str) -> np.ndarray:
        if name == "tsdf":
            out = np.empty(2 * self.R ** 3, np.float32)
        elif name == "dist":
            out = np.empty(self.W * self.H, np.float32)
        elif name == "flags":
            out = np.empty((self.R // 8) ** 3, np.uint8)
        else:
            out = np.empty(4 * self.W * self.H, np.float32)
        check(lib().recon_tsdf_get(self.h, name.encode(), _ptr(out), out.nbytes))
        return out

    def set_grid(self, grid):
        self._inputs_ready(grid)
        check(lib().recon_tsdf_set_grid(self.h, _ptr(grid), _on_device(grid)))

    def enable_timing(self, on: bool = True):
        check(lib().recon_tsdf_enable_timing(self.h, int(on)))

    def timing(self, reset: bool = True) -> dict:
        ms = np.zeros(5, np.float64)
        n = np.zeros(5, np.int64)
        check(lib().recon_tsdf_get_timing(self.h, _ptr(ms), _ptr(n), int(reset)))
        return {k: (float(ms[i]), int(n[i])) for i, k in enumerate(TSDF_TIMING_KINDS)}

    def enable_counting(self, on: bool = True):
        check(lib().recon_tsdf_enable_counting(self.h, int(on)))

    def counts(self, reset: bool = True) -> np.ndarray:
        c = np.zeros(3, np.int64)
        check(lib().recon_tsdf_get_counts(self.h, _ptr(c), int(reset)))
        return c


# ---- result files (ResultTxt, TrackingParams) ----

class Trajectory:
    """ResultTxt: poses added one per frame, saved canonized (relative to the
    first) in the reference's text format.  add_identity starts the list with
    the identity, as ResultTxt::init(fn, true) does (main.cpp:1189)."""

    def __init__(self, add_identity: bool = True):
        self.poses = [np.eye(4, dtype=np.float32)] if add_identity else []

    def add_pose(self, T):
        self.poses.append(np.asarray(T, np.float32).reshape(4, 4).copy())

    def save(self, path: str, transpose: int = 1, inverse: int = 0):
        P = np.ascontiguousarray(np.stack(self.poses) if self.poses else np.zeros((0, 4, 4), np.float32), np.float32)
        check(lib().recon_trajectory_save(os.fsencode(path), _ptr(P), len(self.poses), transpose, inverse))


def load_trajectory(path: str, transpose: int = 1, max_poses: int = 10000) -> np.ndarray:
    out = np.zeros((max_poses, 4, 4), np.float32)
    n = check(lib().recon_trajectory_load(os.fsencode(path), _ptr(out), max_poses, transpose))
    return out[:n]


def load_track_params(path: str, max_n: int = 100000):
    """TrackingParams::init: [(frame, mode, lambda)] of a mode file."""
    fr = np.zeros(max_n, np.int32)
    md = np.zeros(max_n, np.int32)
    la = np.zeros(max_n, np.float32)
    n = check(lib().recon_track_params_load(os.fsencode(path), _ptr(fr), _ptr(md), _ptr(la), max_n))
    n = min(n, max_n)
    return [(int(fr[i]), int(md[i]), float(la[i])) for i in range(n)]


def track_params_for(params, frame: int):
    """TrackingParams::getParams: the entry nearest to `frame` (the first on
    ties); (frame, GEOMETRIC, 1.0)-like default when there are none."""
    if not params:
        return (frame, GEOMETRIC, 1.0)
    fr = np.ascontiguousarray([p[0] for p in params], np.int32)
    return params[lib().recon_track_params_lookup(_ptr(fr), len(params), frame)]


# ---- Kinect pre-processing (include/recon_kinect.h); torch CUDA tensors in and out ----

def _stream_now():
    import torch
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def kinect_disparity_to_depth(disp, c0: float, c1: float, min_dist: float, max_dist: float, x_off: float = 0.0,
                              y_off: float = 0.0, half_resolution: bool = False, out=None):
    """OMPFunctions::d2Z / d2ZLow on the GPU: uint16 disparity [H, W] (a CUDA
    tensor, int16 or uint16 storage) -> float depth in mm, on torch's current stream."""
    import torch
    H, W = disp.shape
    shape = (H // 2, W // 2) if half_resolution else (H, W)
    if out is None:
        out = torch.empty(shape, dtype=torch.float32, device=disp.device)
    check(lib().recon_kinect_disparity_to_depth(_ptr(disp), W, H, c0, c1, min_dist, max_dist, x_off, y_off,
                                                int(half_resolution), _ptr(out), _stream_now()))
    return out


def kinect_rgb_to_gray(rgb, out=None):
    """OMPFunctions::convert2Gray on the GPU: uint8 [H, W, 3] -> uint8 [H, W]."""
    import torch
    H, W = rgb.shape[:2]
    if out is None:
        out = torch.zeros((H, W), dtype=torch.uint8, device=rgb.device)
    check(lib().recon_kinect_rgb_to_gray(_ptr(rgb), W, H, _ptr(out), _stream_now()))
    return out


def kinect_undistort_gray(src, K, iK, kc, out=None):
    """OMPFunctions::undistort (lookup form) on the GPU: uint8 [H, W] -> uint8 [H, W]."""
    import torch
    H, W = src.shape
    if out is None:
        out = torch.zeros((H, W), dtype=torch.uint8, device=src.device)
    Kf = np.ascontiguousarray(np.asarray(K, np.float32).reshape(9))
    iKf = np.ascontiguousarray(np.asarray(iK, np.float32).reshape(9))
    kcf = np.ascontiguousarray(np.asarray(kc, np.float32).reshape(-1)[:5])
    check(lib().recon_kinect_undistort_gray(_ptr(src), W, H, _ptr(Kf), _ptr(iKf), _ptr(kcf), _ptr(out), _stream_now()))
    return out


# the reference's GPU capture path (d2z.cu, rgb2gray.cu, undistort.cu)

def kinect_disparity_to_float(disp, out=None):
    """undistortDisparityCuda: uint16 disparity [H, W] -> float, 65535 where >= 2047."""
    import torch
    H, W = disp.shape
    if out is None:
        out = torch.empty((H, W), dtype=torch.float32, device=disp.device)
    check(lib().recon_kinect_disparity_to_float(_ptr(disp), W, H, _ptr(out), _stream_now()))
    return out


def kinect_depth_normalized(disp, c0: float, c1: float, min_dist: float, max_dist: float, x_off: float = 0.0,
                            y_off: float = 0.0, out=None):
    """d2ZCuda (16-bit disparity) / d2ZCudaHdr (float disparity): [H, W] ->
    the [H/2, W/2] depth normalised by (z - min_dist) / (max_dist - min_dist)."""
    import torch
    H, W = disp.shape
    if out is None:
        out = torch.empty((H // 2, W // 2), dtype=torch.float32, device=disp.device)
    is_f = disp.dtype == torch.float32
    check(lib().recon_kinect_depth_normalized(None if is_f else _ptr(disp), _ptr(disp) if is_f else None, W, H, c0, c1,
                                              min_dist, max_dist, x_off, y_off, _ptr(out), _stream_now()))
    return out


def kinect_rgb_to_hdr(rgb, out=None):
    """convertToHDRCuda: uint8 [H, W, 3] -> float [H, W, 3], every byte / 255."""
    import torch
    H, W = rgb.shape[:2]
    if out is None:
        out = torch.empty((H, W, 3), dtype=torch.float32, device=rgb.device)
    check(lib().recon_kinect_rgb_to_hdr(_ptr(rgb), W, H, _ptr(out), _stream_now()))
    return out


def kinect_rgb_to_gray_hdr(rgb, out=None):
    """rgb2GrayCuda: uint8 [H, W, 3] (integer weights) or float [H, W, 3]
    (0.3 r + 0.59 g + 0.11 b) -> float gray [H, W]."""
    import torch
    H, W = rgb.shape[:2]
    if out is None:
        out = torch.empty((H, W), dtype=torch.float32, device=rgb.device)
    is_f = rgb.dtype == torch.float32
    check(lib().recon_kinect_rgb_to_gray_hdr(None if is_f else _ptr(rgb), _ptr(rgb) if is_f else None, W, H, _ptr(out),
                                             _stream_now()))
    return out


def kinect_undistort_rgb_hdr(rgb, K, iK, kc, out=None):
    """undistortRGBCuda: uint8 [H, W, 3] -> undistorted float RGB [H, W, 3]."""
    import torch
    H, W = rgb.shape[:2]
    if out is None:
        out = torch.empty((H, W, 3), dtype=torch.float32, device=rgb.device)
    Kf = np.ascontiguousarray(np.asarray(K, np.float32).reshape(9))
    iKf = np.ascontiguousarray(np.asarray(iK, np.float32).reshape(9))
    kcf = np.ascontiguousarray(np.asarray(kc, np.float32).reshape(-1)[:5])
    check(lib().recon_kinect_undistort_rgb_hdr(_ptr(rgb), W, H, _ptr(Kf), _ptr(iKf), _ptr(kcf), _ptr(out),
                                               _stream_now()))
    return out
