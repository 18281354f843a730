"""The filtered reference: ICP points and normals from the ray cast of a fused
TSDF (genOrientedPoints6Kernel, d2z.cu:471-501; PhotoTracker::setReferencePoints
with setFilteredReference(true)).

CPU: the oracle's oriented points are the reference kernel's bit for bit, and
a tracker on a filtered keyframe converges to the rendering pose.  GPU: the
ray cast stays on the device and feeds the tracker; the pose is bit-identical
to the oracle's given the same ray-cast images.
"""
import numpy as np
import pytest

import oracle_lib as O
import ref_lib as RL
from recon_gb300 import synth
from scenes import depth_sequence

ROOM = ((0.0, 150.0, -2350.0), (1750.0, 1750.0, 1750.0))


def fused_keyframe(W, H, R, n=5, seed=5):
    """A keyframe (frame 0) and n - 1 neighbours fused into a TSDF by the
    oracle, its ray cast and shading from the keyframe's pose, and a current
    frame 5 frames later."""
    s = depth_sequence(W, H, n + 5, seed=seed, noise=0.001)
    o = O.OracleTSDF(O.tsdf_params(R, W, H, origin=ROOM[0], dim=ROOM[1]))
    for f in range(n):
        o.update(s.dist[f], s.poses[f], s.K)
    xyz = o.raycast(s.poses[0], s.K)
    _, nrm = o.shade(xyz)
    return s, o, xyz, nrm


def grays(s, frames, seed=5):
    sc = synth.make_scene(seed)
    out = []
    for f in frames:
        g, _ = O.render_pair(sc, synth.camera_struct(s.cal, "L", s.poses[f]),
                             synth.camera_struct(s.cal, "R", s.poses[f]), noise_rel=0.001, noise_seed=seed + 1,
                             frame=f)
        out.append(g)
    return out


@pytest.mark.skipif(not RL.available(), reason="oracle/_ref not built (reference tree absent)")
def test_oriented_points_match_reference_kernel():
    W, H = 160, 120
    s, o, xyz, nrm = fused_keyframe(W, H, 128)
    pts_o = np.zeros(6 * W * H, np.float32)
    m_o = np.zeros(W * H, np.int32)
    pts_r = np.zeros_like(pts_o)
    m_r = np.zeros_like(m_o)
    O.lib().orc_gen_oriented_points6(O.ptr(xyz), O.ptr(nrm), W, H, O.ptr(pts_o), O.ptr(m_o))
    cal = np.ascontiguousarray(s.cal.calib, np.float32)
    RL.lib().ref_genOrientedPoints6(O.ptr(xyz), O.ptr(nrm), W, H, O.ptr(cal), O.ptr(pts_r), O.ptr(m_r))
    assert np.array_equal(pts_o.view(np.uint32), pts_r.view(np.uint32)) and np.array_equal(m_o, m_r)
    assert m_o.mean() > 0.3


def test_filtered_reference_tracks_to_rendering_pose():
    W, H = 160, 120
    s, o, xyz, nrm = fused_keyframe(W, H, 128)
    g = grays(s, [0, 5])
    cfg = O.make_config(W, H, 3, mode=O.BIOBJECTIVE, iters=(5, 5, 8), n_select=4096)
    t = O.OracleTracker(cfg, s.cal.calib)
    t.set_reference_oriented(g[0], s.depth[0], xyz, nrm)
    t.set_current(g[1], s.depth[5])
    T, _ = t.track()
    T_gt = synth.relative_pose(s.poses[0].astype(np.float64), s.poses[5].astype(np.float64))
    mm, deg = synth.pose_error(T.astype(np.float64), T_gt)
    assert mm < 5.0 and deg < 0.2, (mm, deg)
    # the ICP reference is the ray cast's, not the raw depth's
    ref6 = t.get("ref6", 0, 6 * W * H, np.float32).reshape(-1, 6)
    mask = t.get("refmask", 0, W * H, np.int32)
    hit = (xyz.reshape(-1, 4)[:, 2] < 0) & (np.linalg.norm(nrm.reshape(-1, 4)[:, :3], axis=1) ** 2 > 1e-7)
    assert np.array_equal(mask.astype(bool), hit)
    np.testing.assert_array_equal(ref6[hit, :3], xyz.reshape(-1, 4)[hit, :3])


@pytest.mark.gpu
def test_filtered_reference_from_device_ray_cast_matches_oracle():
    import recon_gb300 as rg
    W, H, R = 160, 120, 128
    s = depth_sequence(W, H, 10, seed=5, noise=0.001)
    g = grays(s, [0, 5])
    v = rg.TSDF(rg.tsdf_params(R, W, H, cube_origin=ROOM[0], cube_dim=ROOM[1]))
    for f in range(5):
        v.set_dist_depth16(s.depth[f])
        v.update(s.poses[f], s.K)
    v.raycast(s.poses[0], s.K)
    cfg = rg.make_config(W, H, 3, mode=rg.BIOBJECTIVE, iters=(5, 5, 8), n_select=4096)
    trk = rg.Tracker(cfg, s.cal.calib)
    import torch
    gd = torch.from_numpy(g[0]).cuda()
    dd = torch.from_numpy(np.ascontiguousarray(s.depth[0]).view(np.int16)).cuda()
    trk.set_reference_oriented(gd, dd, v.view("xyz"), v.view("normal"))
    trk.set_current(g[1], s.depth[5])
    T, st = trk.track()
    xyz, nrm = v.get("xyz"), v.get("normal")
    ocfg = O.make_config(W, H, 3, mode=O.BIOBJECTIVE, iters=(5, 5, 8), n_select=4096)
    o = O.OracleTracker(ocfg, s.cal.calib)
    o.set_reference_oriented(g[0], s.depth[0], xyz, nrm)
    o.set_current(g[1], s.depth[5])
    To, _ = o.track()
    assert np.array_equal(T.view(np.uint32), To.view(np.uint32)), (T, To)
    pts = trk.get_array(0, "ref_pts", 0, np.float32, 4 * W * H).reshape(-1, 4)
    ref6 = o.get("ref6", 0, 6 * W * H, np.float32).reshape(-1, 6)
    assert np.array_equal(pts[:, :3].view(np.uint32), ref6[:, :3].view(np.uint32))
    # host copies of the same maps give the same reference
    trk2 = rg.Tracker(cfg, s.cal.calib)
    trk2.set_reference_oriented(g[0], s.depth[0], xyz.reshape(H, W, 4), nrm.reshape(H, W, 4))
    trk2.set_current(g[1], s.depth[5])
    T2, _ = trk2.track()
    assert np.array_equal(T2.view(np.uint32), T.view(np.uint32))
    trk.close()
    trk2.close()
    v.close()
