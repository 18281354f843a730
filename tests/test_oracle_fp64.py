"""The FP64 oracle (oracle/oracle_fp64.c) against the FP32 oracle, and the
keyframe colour fusion of the FP32 oracle (CPU only).

The FP64 oracle is the judge of pose error: the same tracker with every
floating-point operation in double and the pose kept in double.  The FP32
oracle (bit-identical to the GPU) must stay well inside the tracking bound of
1 mm / 0.05 deg of it; the tolerance asserted here is 20x tighter than that
bound (0.05 mm / 0.0025 deg).
"""
import numpy as np
import pytest

import oracle_lib as O
from recon_gb300 import synth
from scenes import frame_pair

TOL_MM, TOL_DEG = 0.05, 0.0025


@pytest.mark.parametrize("W,H,mode,seed,distortion", [
    (320, 240, O.PHOTOMETRIC, 3, False),
    (320, 240, O.BIOBJECTIVE, 11, False),
    (320, 240, O.GEOMETRIC, 5, False),
    (640, 480, O.BIOBJECTIVE, 3, True),
])
def test_fp32_oracle_within_tolerance_of_fp64(W, H, mode, seed, distortion):
    p = frame_pair(W, H, seed=seed, distortion=distortion)
    it = (1, 3, 10, 5) if W == 640 else (10, 10, 10)
    cfg = O.make_config(W, H, p.L, mode=mode, iters=it)
    o32 = O.OracleTracker(cfg, p.cal.calib)
    o32.set_reference(p.g0, p.d0)
    o32.set_current(p.g1, p.d1)
    T32, _ = o32.track()
    o64 = O.Oracle64Tracker(cfg, p.cal.calib)
    o64.set_reference(p.g0, p.d0)
    o64.set_current(p.g1, p.d1)
    T64 = o64.track()
    mm, deg = synth.pose_error(T32.astype(np.float64), T64)
    assert mm < TOL_MM and deg < TOL_DEG, (mm, deg)
    # with a photometric term both converge to the rendering pose within the
    # noise of the data (point-to-plane ICP alone slides along this scene's planes)
    if mode != O.GEOMETRIC:
        mm_gt, deg_gt = synth.pose_error(T64, p.T_gt)
        assert mm_gt < 5.0 and deg_gt < 0.2, (mm_gt, deg_gt)
    # the FP64 selection is the FP32 one up to points whose gradient bin flips
    s32 = o32.get("sel_idx", 0, cfg.n_select, np.int32)
    s64 = o64.get("sel_idx", 0, cfg.n_select, np.int32)
    assert len(np.intersect1d(s32, s64)) >= 0.99 * cfg.n_select


def test_fp64_oracle_does_not_depend_on_thread_count():
    p = frame_pair(320, 240, seed=9)
    cfg = O.make_config(320, 240, 3, mode=O.BIOBJECTIVE, iters=(3, 3, 3))
    out = []
    for threads in (1, O.lib().orc_num_threads()):
        O.lib().orc_set_threads(threads)
        o = O.Oracle64Tracker(cfg, p.cal.calib)
        o.set_reference(p.g0, p.d0)
        o.set_current(p.g1, p.d1)
        out.append(o.track())
    O.lib().orc_set_threads(0)
    assert np.array_equal(out[0].view(np.uint64), out[1].view(np.uint64))


def _segment(W, H, n, seed):
    cal = synth.make_calibration(W, H)
    sc = synth.make_scene(seed)
    poses = synth.smooth_trajectory(n, seed + 2)
    g, d = [], []
    for f in range(n):
        gf, df = O.render_pair(sc, synth.camera_struct(cal, "L", poses[f]), synth.camera_struct(cal, "R", poses[f]),
                               noise_rel=0.01, noise_seed=seed + 1, frame=f)
        g.append(gf)
        d.append(df)
    return cal, poses, g, d


def test_fp64_fusion_agrees_with_fp32_fusion():
    """Depth and colour fusion of five tracked frames: the FP64 oracle's fused
    keyframe and the poses tracked against it agree with the FP32 oracle's."""
    W, H = 320, 240
    cal, poses, g, d = _segment(W, H, 8, seed=81)
    cfg = O.make_config(W, H, 3, mode=O.BIOBJECTIVE, iters=(2, 3, 4))
    o32 = O.OracleTracker(cfg, cal.calib)
    o64 = O.Oracle64Tracker(cfg, cal.calib)
    o32.set_reference(g[0], d[0])
    o64.set_reference(g[0], d[0])
    T32, T64, T32s, T64s = None, None, [], []
    for f in range(1, 6):
        o32.set_current(g[f], d[f])
        o64.set_current(g[f], d[f])
        T32, _ = o32.track(T32)
        T64 = o64.track(T64)
        T32s.append(T32.copy())
        T64s.append(T64.copy())
    o32.fuse_keyframe([d[f] for f in range(1, 6)], np.stack(T32s), gate=30.0, grays=[g[f] for f in range(1, 6)])
    o64.fuse_keyframe([d[f] for f in range(1, 6)], np.stack(T64s), gate=30.0, grays=[g[f] for f in range(1, 6)])
    z32 = o32.get("ref_z", 0, W * H, np.float32).astype(np.float64)
    z64 = o64.get("ref_z", 0, W * H, np.float64)
    agree = np.abs(z32 - z64) < 0.01
    assert agree.mean() > 0.995, agree.mean()  # a gate decision may flip on a handful of pixels
    c32 = o32.get("ref_col", 0, W * H, np.float32).astype(np.float64)
    c64 = o64.get("ref_col", 0, W * H, np.float64)
    assert np.array_equal(c32 < 0, c64 < 0) or (np.mean((c32 < 0) != (c64 < 0)) < 0.005)
    both = (c32 >= 0) & (c64 >= 0)
    assert np.mean(np.abs(c32[both] - c64[both]) < 1e-4) > 0.995
    for f in (6, 7):
        o32.set_current(g[f], d[f])
        o64.set_current(g[f], d[f])
        T32, _ = o32.track(T32)
        T64 = o64.track(T64)
        mm, deg = synth.pose_error(T32.astype(np.float64), T64)
        assert mm < TOL_MM and deg < TOL_DEG, (f, mm, deg)


def test_colour_fusion_properties():
    """orc_fuse_rgbd on a keyframe and frames seen from the same pose: every
    frame passes the gate, the fused depth is the mean of equal values and the
    fused colour is the keyframe's own sample; a frame 100 mm away fails the
    gate and changes nothing."""
    W, H = 320, 240
    p = frame_pair(W, H, seed=21)
    L = O.lib()
    n = W * H
    z = np.zeros(n, np.float32)
    gk = np.zeros(n, np.float32)
    d0 = np.ascontiguousarray(p.d0.reshape(-1))
    g0 = np.ascontiguousarray(p.g0.reshape(-1))
    L.orc_convert_depth(O.ptr(d0), n, O.ptr(z))
    L.orc_convert_gray(O.ptr(g0), n, O.ptr(gk))
    eye = np.tile(np.eye(4, dtype=np.float32).reshape(16), 3)
    cal = np.ascontiguousarray(p.cal.calib, np.float32)

    def fuse(zs, gs):
        zo = np.zeros(n, np.float32)
        wo = np.zeros(n, np.float32)
        co = np.zeros(n, np.float32)
        L.orc_fuse_rgbd(O.ptr(z), O.ptr(gk), W, H, O.ptr(cal), len(zs), O.ptrs(zs), O.ptrs(gs), O.ptr(eye), 30.0,
                        O.ptr(zo), O.ptr(wo), O.ptr(co))
        return zo, wo, co

    zo, wo, co = fuse([z, z, z], [gk, gk, gk])
    valid = (z < -cal[62]) & (z > -cal[63])
    assert np.all(wo[valid] == 4.0) and np.all(wo[~valid] == 0.0)
    np.testing.assert_allclose(zo[valid], z[valid], rtol=1e-6)
    has = co >= 0
    assert has[valid].mean() > 0.9 and not has[~valid].any()
    # the mean of four equal samples is the keyframe's own sample, xyz2CloudKernel's color1
    # (to the float rounding of the point: the fusion forms it with reciprocals
    # of fx, fy and the depth where xyz2CloudKernel's inputs divide)
    xyz = np.zeros(4 * n, np.float32)
    L.orc_zmap_to_xyz(O.ptr(z), W, H, O.ptr(cal), O.ptr(xyz))
    vdata = np.zeros(24 * n, np.float32)
    L.orc_xyz2cloud(O.ptr(xyz), W, H, O.ptr(cal), O.ptr(gk), O.ptr(vdata))
    col1 = vdata.reshape(n, 24)[:, 14]
    inb = vdata.reshape(n, 24)[:, 2] < 0
    inb &= vdata.reshape(n, 24)[:, 6] != 0
    np.testing.assert_allclose(co[inb], col1[inb], rtol=2e-5, atol=1e-6)
    # a frame whose depth is 100 mm off fails the 30 mm gate
    zfar = np.where(z != 0, z - 100.0, 0.0).astype(np.float32)
    zo2, wo2, co2 = fuse([zfar], [gk])
    assert np.all(wo2[valid] == 1.0)
    np.testing.assert_array_equal(zo2[valid], z[valid])
