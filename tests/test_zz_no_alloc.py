"""The allocation-free photometric iteration (recon_photometric_iteration_noalloc).

Callers that cannot allocate device memory while tracking (a real-time frame
loop where cudaMalloc could stall the frame, a host framework that owns all
device memory) use this entry point: its scratch is a fixed array inside the
library.  The test calls it through the C ABI twice in a row, with the pose
updated in place on the device, and requires the same poses, bit for bit, as
the first two photometric iterations of the regular batch entry point on the
same inputs.  This file is collected last so that a run that stops at the first
failure has run every other test before it.
"""
import ctypes

import numpy as np
import pytest

import recon_gb300 as rg
from scenes import frame_pair

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


class PhotoView(ctypes.Structure):
    """recon_photo_view (include/recon_track.h)."""
    _fields_ = [
        ("n_points", ctypes.c_int32), ("level", ctypes.c_int32),
        ("img_width", ctypes.c_int32), ("img_height", ctypes.c_int32),
        ("depth_width", ctypes.c_int32), ("depth_height", ctypes.c_int32),
        ("hist_bins", ctypes.c_int32), ("solver", ctypes.c_int32), ("opt_scale_out", ctypes.c_float),
        ("calib", ctypes.c_float * 96),
        ("xyz", ctypes.c_void_p), ("intensity", ctypes.c_void_p), ("jacobian", ctypes.c_void_p),
        ("img", ctypes.c_void_p), ("depth", ctypes.c_void_p),
    ]


def _noalloc():
    L = rg.lib()
    f = L.recon_photometric_iteration_noalloc
    f.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    f.restype = ctypes.c_int32
    return f


@pytest.mark.parametrize("level,solver,P", [(1, rg.SOLVER_CHOLESKY, 8192), (0, rg.SOLVER_CG, 8192),
                                            (0, rg.SOLVER_CHOLESKY, 16384)])
def test_noalloc_iterations_match_batch_entry_point(level, solver, P):
    """P = 16384 is the largest size the built-in array holds (both of its
    halves used to the end)."""
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    W, H, L = 320, 240, 3
    p = frame_pair(W, H, seed=61)
    iters = [0, 0, 0]
    iters[L - 1 - level] = 2
    cfg = rg.make_config(W, H, L, mode=rg.PHOTOMETRIC, iters=iters, n_select=P, solver=solver)
    trk = rg.Tracker(cfg, p.cal.calib)
    trk.enable_trace(8)
    trk.set_reference(p.g0, p.d0)
    trk.set_current(p.g1, p.d1)
    T_batch, _ = trk.track()
    trace = trk.trace(0)
    assert len(trace) == 2

    wl, hl = W >> level, H >> level
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    xyz = dev(trk.get_array(0, "sel_xyz", 0, np.float32, 3 * P))
    inten = dev(trk.get_array(0, "sel_I", level, np.float32, P))
    jac = dev(trk.get_array(0, "sel_J", level, np.float32, 6 * P))
    img = dev(trk.get_array(0, "cur_gray", level, np.float32, wl * hl))
    depth = dev(trk.get_array(0, "cur_z", 0, np.float32, W * H))
    T = torch.eye(4, dtype=torch.float32, device="cuda").contiguous()

    v = PhotoView()
    v.n_points, v.level = P, level
    v.img_width, v.img_height, v.depth_width, v.depth_height = wl, hl, W, H
    v.hist_bins, v.solver, v.opt_scale_out = 64, solver, 1e3
    v.calib[:] = p.cal.calib.tolist()
    v.xyz, v.intensity, v.jacobian = xyz.data_ptr(), inten.data_ptr(), jac.data_ptr()
    v.img, v.depth = img.data_ptr(), depth.data_ptr()

    f = _noalloc()
    for k in range(2):
        rc = f(ctypes.byref(v), ctypes.c_void_p(T.data_ptr()), None)
        assert rc == 0, rg.lib().recon_last_error().decode()
        torch.cuda.synchronize()
        got = T.cpu().numpy().reshape(-1)
        want = np.array(trace[k].T, np.float32)
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), (k, got, want)
    assert np.array_equal(T.cpu().numpy().view(np.uint32), T_batch.view(np.uint32))


def test_noalloc_rejects_too_many_points():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    v = PhotoView()
    v.n_points = 16384 + 1024
    v.level, v.img_width, v.img_height, v.depth_width, v.depth_height = 0, 320, 240, 320, 240
    v.hist_bins, v.solver, v.opt_scale_out = 64, 0, 1e3
    buf = torch.zeros(1 << 20, dtype=torch.float32, device="cuda")
    v.xyz = v.intensity = v.jacobian = v.img = v.depth = buf.data_ptr()
    T = torch.eye(4, dtype=torch.float32, device="cuda").contiguous()
    rc = _noalloc()(ctypes.byref(v), ctypes.c_void_p(T.data_ptr()), None)
    assert rc == -1
    assert b"RECON_NOALLOC_MAX_POINTS" in rg.lib().recon_last_error()
