"""The single tracker's host pose bookkeeping, the keyframe trigger and the
tracker's behaviour on degenerate inputs, on the GPU.

* recon_track's relative and global poses follow PhotoTracker::applyIncrement
  (phototracker.cpp:514-531) bit for bit (pose_book.apply_increment_ref_order,
  itself pinned to the reference's code).
* The keyframe trigger (referenceOutdated, phototracker.cpp:290-296).
* Faults made on the host, none of which faults the GPU: a texture-less frame,
  a start pose that sees nothing, a current frame without depth, NaN depth in
  the reference's float4 input.  Each frame reports its status
  (RECON_ERR_NON_SPD, RECON_ERR_NOT_ENOUGH_POINTS) and keeps its pose, and
  the pose equals the oracle's where the oracle runs the same input.
"""
import numpy as np
import pytest

import oracle_lib as O
import recon_gb300 as rg
from pose_book import apply_increment_ref_order
from recon_gb300 import synth
from scenes import frame_pair

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module", autouse=True)
def cuda_lib():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    rg.lib()


def _frames(W, H, n, seed):
    cal = synth.make_calibration(W, H)
    sc = synth.make_scene(seed)
    poses = synth.smooth_trajectory(n, seed + 2)
    out = []
    for f in range(n):
        out.append(O.render_pair(sc, synth.camera_struct(cal, "L", poses[f]), synth.camera_struct(cal, "R", poses[f]),
                                 noise_rel=0.01, noise_seed=seed + 1, frame=f))
    return cal, out


def bits(a):
    a = np.ascontiguousarray(a)
    return a.view(np.uint32) if a.dtype == np.float32 else a.view(np.uint64)


def test_global_pose_follows_apply_increment():
    W, H = 320, 240
    cal, fr = _frames(W, H, 8, seed=61)
    cfg = rg.make_config(W, H, 3, mode=rg.BIOBJECTIVE, iters=(2, 3, 4))
    trk = rg.Tracker(cfg, cal.calib)
    trk.set_reference(*fr[0])
    T_host = np.eye(4, dtype=np.float32)
    G = np.eye(4)
    assert np.array_equal(trk.global_pose(), G) and np.array_equal(trk.relative_pose(), T_host)
    for f in range(1, 8):
        if f == 5:
            # a new keyframe: the relative pose restarts at the identity, the global pose is kept
            trk.set_reference(*fr[4])
            T_host = np.eye(4, dtype=np.float32)
            assert np.array_equal(trk.relative_pose(), T_host)
        trk.set_current(*fr[f])
        Trel, st = trk.track()
        assert st.status == rg.OK
        T_host, G = apply_increment_ref_order(T_host, G, Trel)
        assert np.array_equal(bits(trk.relative_pose()), bits(T_host)), f
        assert np.array_equal(bits(trk.global_pose()), bits(G)), f
    trk.reset()
    assert np.array_equal(trk.global_pose(), np.eye(4)) and np.array_equal(trk.relative_pose(), np.eye(4))
    trk.close()


def test_reference_outdated_trigger():
    W, H = 320, 240
    cal, fr = _frames(W, H, 2, seed=62)
    cfg = rg.make_config(W, H, 3, mode=rg.PHOTOMETRIC, iters=(0, 0, 0))
    trk = rg.Tracker(cfg, cal.calib)
    assert trk.reference_outdated()  # no reference yet
    trk.set_reference_updating(True, 125.0, 12.5)
    trk.set_reference(*fr[0])
    trk.set_current(*fr[1])
    assert not trk.reference_outdated()
    # with no iterations the tracked pose is the start pose: far enough to trigger
    for deg, mm, want in ((2.0, 20.0, False), (5.0, 130.0, True), (13.0, 10.0, True)):
        trk.set_reference(*fr[0])
        Tstart = synth.offset_pose(3, deg, mm).astype(np.float32)
        trk.track(Tstart)
        assert trk.reference_outdated() == want, (deg, mm)
        assert trk.reference_outdated() == rg.pose_difference_exceeded(trk.relative_pose(), 125.0, 12.5)
    trk.set_reference_updating(False)
    assert not trk.reference_outdated()
    trk.close()
    # the batch form tests each instance's tracked pose
    b = rg.Batch([cfg, cfg], [cal.calib, cal.calib])
    b.set_reference([fr[0][0]] * 2, [fr[0][1]] * 2)
    b.set_current([fr[1][0]] * 2, [fr[1][1]] * 2)
    T0 = np.stack([synth.offset_pose(3, 1.0, 10.0), synth.offset_pose(3, 1.0, 200.0)]).astype(np.float32)
    T, _ = b.track(T0)
    assert b.reference_outdated().tolist() == [False, True]
    b.close()


def _oracle_track(cfg_args, cal, ref, cur, T0=None, ref_float=None):
    orc = O.OracleTracker(O.make_config(*cfg_args[0], **cfg_args[1]), cal.calib)
    if ref_float is not None:
        orc.set_reference_float(*ref_float)
    else:
        orc.set_reference(*ref)
    orc.set_current(*cur)
    To, _ = orc.track(T0)
    orc.close()
    return To


def test_textureless_reference_rejects_the_solve_and_keeps_the_pose():
    p = frame_pair(320, 240, seed=63)
    flat = np.full_like(p.g0, 128)
    args = ((320, 240, 3), dict(mode=O.PHOTOMETRIC, iters=(2, 2, 2)))
    trk = rg.Tracker(rg.make_config(320, 240, 3, mode=rg.PHOTOMETRIC, iters=(2, 2, 2)), p.cal.calib)
    trk.set_reference(flat, p.d0)
    trk.set_current(p.g1, p.d1)
    T0 = synth.offset_pose(5, 1.0, 5.0).astype(np.float32)
    T, st = trk.track(T0)
    assert st.status == rg.ERR_NON_SPD and st.non_spd == st.iterations == 6
    assert np.allclose(T, T0, atol=1e-5)  # the rejected solves leave the pose (renormalised) where it was
    assert np.array_equal(bits(T), bits(_oracle_track(args, p.cal, (flat, p.d0), (p.g1, p.d1), T0)))
    trk.close()


def test_start_pose_that_sees_nothing():
    p = frame_pair(320, 240, seed=64)
    away = np.eye(4, dtype=np.float32)
    away[0, 3] = 20000.0  # 20 m to the side: every point projects far outside the image
    for mode, want in ((rg.PHOTOMETRIC, rg.ERR_NON_SPD), (rg.GEOMETRIC, rg.ERR_NOT_ENOUGH_POINTS),
                       (rg.BIOBJECTIVE, rg.ERR_NOT_ENOUGH_POINTS)):
        trk = rg.Tracker(rg.make_config(320, 240, 3, mode=mode, iters=(1, 1, 1)), p.cal.calib)
        trk.set_reference(p.g0, p.d0)
        trk.set_current(p.g1, p.d1)
        T, st = trk.track(away)
        assert st.status == want, (mode, st.status)
        assert np.all(np.isfinite(T)) and abs(T[0, 3] - 20000.0) < 1e-2
        args = ((320, 240, 3), dict(mode=mode, iters=(1, 1, 1)))
        assert np.array_equal(bits(T), bits(_oracle_track(args, p.cal, (p.g0, p.d0), (p.g1, p.d1), away))), mode
        trk.close()


def test_current_frame_without_depth():
    p = frame_pair(320, 240, seed=65)
    nodepth = np.zeros_like(p.d1)
    T0 = synth.offset_pose(6, 0.5, 5.0).astype(np.float32)
    for mode in (rg.GEOMETRIC, rg.BIOBJECTIVE):
        trk = rg.Tracker(rg.make_config(320, 240, 3, mode=mode, iters=(2, 2, 2)), p.cal.calib)
        trk.set_reference(p.g0, p.d0)
        trk.set_current(p.g1, nodepth)
        T, st = trk.track(T0)
        assert st.status == rg.ERR_NOT_ENOUGH_POINTS and st.solves == 0
        assert list(st.icp_selected)[:3] == [0, 0, 0]
        assert np.array_equal(bits(T), bits(T0))  # no solve ran: the pose is the start pose
        trk.close()


def test_nan_depth_in_float4_reference():
    """The reference's float4 RGBA + normalised-depth frame with NaN depth on a
    quarter of the pixels: those pixels are invalid, tracking runs on the rest
    and equals the oracle given the same converted frame."""
    p = frame_pair(320, 240, seed=66)
    W, H = 320, 240
    cal = p.cal.calib
    mind, maxd = float(cal[62]), float(cal[63])
    g = p.g0.astype(np.float32) / 255.0
    depth = p.d0.astype(np.float32)
    w = np.where(p.d0 > 0, (depth - mind) / (maxd - mind), -1.0).astype(np.float32)
    w[::2, ::2] = np.nan
    rgbd = np.zeros((H, W, 4), np.float32)
    rgbd[..., 0] = rgbd[..., 1] = rgbd[..., 2] = g
    rgbd[..., 3] = w
    rgbd = np.ascontiguousarray(rgbd[::-1])  # rows stored bottom-up
    trk = rg.Tracker(rg.make_config(W, H, 3, mode=rg.BIOBJECTIVE, iters=(2, 3, 4)), cal)
    trk.set_reference_rgbd_float4(0, rgbd)
    trk.set_current(p.g1, p.d1)
    T, st = trk.track()
    assert st.status == rg.OK and np.all(np.isfinite(T))
    gz = np.zeros(W * H, np.float32)
    zz = np.zeros(W * H, np.float32)
    calc = np.ascontiguousarray(cal, np.float32)
    O.lib().orc_rgbd_float4_to_gray_z(O.ptr(rgbd), W, H, O.ptr(calc), O.ptr(gz), O.ptr(zz))
    assert np.isnan(zz).sum() == (H // 2) * (W // 2)
    args = ((W, H, 3), dict(mode=O.BIOBJECTIVE, iters=(2, 3, 4)))
    To = _oracle_track(args, p.cal, None, (p.g1, p.d1), ref_float=(gz, zz))
    assert np.array_equal(bits(T), bits(To))
    mm, deg = synth.pose_error(T.astype(np.float64), p.T_gt)
    assert mm < 5.0 and deg < 0.2, (mm, deg)
    trk.close()
