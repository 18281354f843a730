"""The reconstruction stream's oracle (oracle/oracle_tsdf.c) on the CPU.

Pinned bit for bit to the reference's own kernels (tracker/kernels/
VoxelGrid_cuda.cu, built for the host by oracle/build_ref.py): reset, update,
ray cast, shading, resampling and the distance map of a float4 RGB-D frame.
Then properties of the fused surface: it reproduces the rendered depth to a
small fraction of a voxel, and a frame fused twice doubles the weights.
"""
import ctypes

import numpy as np
import pytest

import oracle_lib as O
import ref_lib as RL
from scenes import depth_sequence

# the reference's grid placement and one that holds the whole synthetic room
CUBES = {
    "reference": (O.TSDF_ORIGIN, O.TSDF_DIM),
    "room": ((0.0, 150.0, -2350.0), (1750.0, 1750.0, 1750.0)),
}

needs_ref = pytest.mark.skipif(not RL.available(), reason="oracle/_ref not built (reference tree absent)")


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


@needs_ref
@pytest.mark.parametrize("cube", sorted(CUBES))
def test_tsdf_oracle_matches_reference_kernels(cube):
    W, H, R = 160, 120, 64
    s = depth_sequence(W, H, 4, seed=5, noise=0.001)
    origin, dim = CUBES[cube]
    p = O.tsdf_params(R, W, H, origin=origin, dim=dim)
    o = O.OracleTSDF(p)
    L = RL.lib()
    ref = np.zeros_like(o.grid)
    L.ref_tsdf_reset(O.ptr(ref), R ** 3)
    assert np.array_equal(bits(ref), bits(o.grid))
    org = np.array(origin, np.float32)
    dm = np.array(dim, np.float32)
    K = s.K
    for f in range(4):
        T = np.ascontiguousarray(s.poses[f].reshape(-1))
        d = np.ascontiguousarray(s.dist[f].reshape(-1))
        o.update(d, T, K)
        L.ref_tsdf_update(O.ptr(ref), R, O.ptr(org), O.ptr(dm), W, H, p.min_dist, p.max_dist, O.ptr(T), O.ptr(K),
                          O.ptr(d))
        assert np.array_equal(bits(ref), bits(o.grid)), f
    assert (o.grid[1::2] > 0).mean() > 0.1 and (o.grid[0::2] < 0).any()
    for f in (0, 3):
        T = np.ascontiguousarray(s.poses[f].reshape(-1))
        for filt in (0, 1):
            xyz = o.raycast(T, K, filtering=bool(filt))
            xr = np.zeros_like(xyz)
            L.ref_tsdf_raycast(O.ptr(ref), R, O.ptr(org), O.ptr(dm), W, H, p.min_dist, p.max_dist, O.ptr(T), O.ptr(K),
                               filt, O.ptr(xr))
            assert np.array_equal(bits(xyz), bits(xr)), (f, filt)
        assert (xyz[3::4] > 0).mean() > 0.005
        sh, nr = o.shade(xyz)
        sr, nrr = np.zeros_like(xyz), np.zeros_like(xyz)
        L.ref_tsdf_shade(O.ptr(xyz), W, H, O.ptr(sr), O.ptr(nrr))
        assert np.array_equal(bits(sh), bits(sr)) and np.array_equal(bits(nr), bits(nrr))
    Tr = np.ascontiguousarray(s.poses[2].reshape(-1))
    rs = o.resampled(Tr)
    rr = np.zeros_like(rs)
    L.ref_tsdf_resample(O.ptr(rr), O.ptr(ref), R, O.ptr(org), O.ptr(dm), O.ptr(Tr))
    assert np.array_equal(bits(rs), bits(rr))


def rgbd_frame(dist, min_dist, max_dist):
    """A float4 RGB-D frame (rows bottom-up, w = normalised depth) of a distance map."""
    H, W = dist.shape
    f = np.zeros((H, W, 4), np.float32)
    z = dist.astype(np.float32)
    w = (z - np.float32(min_dist)) / (np.float32(max_dist) - np.float32(min_dist))
    w[z == 0] = 0.0
    f[..., 3] = w[::-1]
    f[..., 0] = 0.25
    return np.ascontiguousarray(f)


@needs_ref
def test_distance_map_of_rgbd_frame_matches_reference():
    W, H = 160, 120
    s = depth_sequence(W, H, 1, seed=8, noise=0.002)
    rgbd = rgbd_frame(s.dist[0], 400.0, 4500.0)
    rgbd[0, :5, 3] = 1.0  # outside (tol, 1 - tol): no depth
    rgbd[1, :5, 3] = 5e-5
    d_o = np.zeros(W * H, np.float32)
    d_r = np.zeros(W * H, np.float32)
    O.lib().orc_tsdf_dist_from_rgbd(O.ptr(rgbd), W, H, 400.0, 4500.0, O.ptr(d_o))
    RL.lib().ref_tsdf_reconstruction(O.ptr(rgbd), W, H, 400.0, 4500.0, O.ptr(d_r))
    assert np.array_equal(bits(d_o), bits(d_r))
    assert (d_o > 0).mean() > 0.5
    assert np.all(d_o.reshape(H, W)[H - 1, :5] == 0) and np.all(d_o.reshape(H, W)[H - 2, :5] == 0)


def test_fused_surface_reproduces_rendered_depth():
    """Six noise-free frames fused into a 128^3 grid: the ray-cast surface seen
    from a fused pose lies within a tenth of a voxel of the rendered depth."""
    W, H, R = 160, 120, 128
    s = depth_sequence(W, H, 6, seed=5, noise=0.0)
    origin, dim = CUBES["room"]
    p = O.tsdf_params(R, W, H, origin=origin, dim=dim)
    o = O.OracleTSDF(p)
    for f in range(6):
        o.update(s.dist[f], s.poses[f], s.K)
    xyz = o.raycast(s.poses[5], s.K).reshape(H, W, 4)
    hit = xyz[..., 3] > 0
    d = s.dist[5]
    both = hit & (d > 0)
    assert both.mean() > 0.5, both.mean()
    voxel = 2 * dim[0] / R
    err = np.abs(-xyz[..., 2][both] - d[both])
    assert np.median(err) < 0.1 * voxel, (np.median(err), voxel)
    assert np.percentile(err, 90) < 0.5 * voxel
    # the ray length is the distance along the unit ray: x, y, z scale together
    ray = np.linalg.norm(xyz[..., :3][both], axis=-1)
    assert np.all(ray > p.min_dist) and np.all(ray < p.max_dist)
    sh, nr = o.shade(xyz.reshape(-1))
    n = nr.reshape(H, W, 4)
    lit = sh.reshape(H, W, 4)[..., 0] > 0
    assert lit.mean() > 0.3
    np.testing.assert_allclose(np.linalg.norm(n[lit][:, :3], axis=-1), 1.0, rtol=1e-5)
    assert np.all(n[lit][:, 2] > 0)


def test_update_running_mean_and_weight_cap():
    """A frame fused k times gives weight min(k, 16) wherever it is fused at
    all, and the tsdf of a voxel fused with the same value stays that value."""
    W, H, R = 80, 60, 32
    s = depth_sequence(W, H, 1, seed=6, noise=0.0)
    p = O.tsdf_params(R, W, H, origin=CUBES["room"][0], dim=CUBES["room"][1])
    o = O.OracleTSDF(p)
    o.update(s.dist[0], s.poses[0], s.K)
    first = o.grid.copy()
    fused = first[1::2] > 0
    assert fused.any() and np.all(first[1::2][fused] == 1.0)
    assert np.all(first[0::2][~fused] == 1.0) and np.all(first[1::2][~fused] == 0.0)
    for k in range(2, 20):
        o.update(s.dist[0], s.poses[0], s.K)
        assert np.all(o.grid[1::2][fused] == min(k, 16)), k
        assert np.all(o.grid[1::2][~fused] == 0.0)
    np.testing.assert_allclose(o.grid[0::2][fused], first[0::2][fused], rtol=0, atol=2e-6)
    assert np.all(np.abs(o.grid[0::2]) <= 1.0)


def test_resample_with_identity_keeps_voxels_inside():
    W, H, R = 80, 60, 32
    s = depth_sequence(W, H, 2, seed=6, noise=0.0)
    p = O.tsdf_params(R, W, H, origin=CUBES["room"][0], dim=CUBES["room"][1])
    o = O.OracleTSDF(p)
    for f in range(2):
        o.update(s.dist[f], s.poses[f], s.K)
    out = o.resampled(np.eye(4, dtype=np.float32)).reshape(R, R, R, 2)
    g = o.grid.reshape(R, R, R, 2)
    # identity: every voxel of index <= R-2 maps onto itself (frac 0)
    np.testing.assert_array_equal(out[:R - 1, :R - 1, :R - 1], g[:R - 1, :R - 1, :R - 1])
    assert np.all(out[R - 1, :, :, 0] == 1.0) and np.all(out[R - 1, :, :, 1] == 0.0)


def test_invert_rt4_is_the_reference_formula():
    rng = np.random.default_rng(3)
    from recon_gb300 import synth
    for _ in range(5):
        T = synth.se3(synth.rodrigues(rng.normal(size=3) * 0.5), rng.normal(size=3) * 500).astype(np.float32)
        Ti = np.zeros(16, np.float32)
        Tf = np.ascontiguousarray(T.reshape(-1))
        O.lib().orc_tsdf_invert_rt4(O.ptr(Tf), O.ptr(Ti))
        np.testing.assert_allclose(Ti.reshape(4, 4) @ T, np.eye(4), atol=2e-4)
        R = T[:3, :3]
        t = T[:3, 3]
        expect = np.float32(0) - (R[0, 0] * t[0] + R[1, 0] * t[1] + R[2, 0] * t[2])
        assert Ti[3] == expect


def edge_case_setup(R=64, W=160, H=120):
    """A camera inside the grid, axis-aligned poses and intrinsics whose
    principal point falls on a pixel centre: the rays of that column / row
    have an exactly zero direction component (the traversal's FLT_MAX
    inverse), and rays start inside the grid (entry parameter 0)."""
    s = depth_sequence(W, H, 3, seed=12, noise=0.0)
    # a wall 1.5 m ahead of the first pose, seen by all three
    s.dist = [np.full((H, W), 1500.0, np.float32) for _ in range(3)]
    K = s.K.copy()
    K[2] = np.float32(80.0) / np.float32(W)  # column 80 looks straight ahead
    K[5] = np.float32(60.0) / np.float32(H)  # row 60 too
    poses = [np.eye(4, dtype=np.float32)]
    Ry = np.eye(4, dtype=np.float32)
    Ry[:3, :3] = np.array([[0, 0, 1], [0, 1, 0], [-1, 0, 0]], np.float32)  # 90 degrees about y
    poses.append(Ry)
    T = np.eye(4, dtype=np.float32)
    T[:3, 3] = [40.0, -25.0, -60.0]
    poses.append(T)
    p = O.tsdf_params(R, W, H, origin=(0.0, 0.0, -1000.0), dim=(1500.0, 1500.0, 1500.0))
    return s, K, poses, p


@needs_ref
def test_traversal_edge_cases_match_reference():
    s, K, poses, p = edge_case_setup()
    W, H, R = p.W, p.H, p.R
    o = O.OracleTSDF(p)
    L = RL.lib()
    ref = np.zeros_like(o.grid)
    L.ref_tsdf_reset(O.ptr(ref), R ** 3)
    org = np.array(p.origin, np.float32)
    dm = np.array(p.dim, np.float32)
    Kc = np.ascontiguousarray(K)
    for f in range(3):
        Tf = np.ascontiguousarray(poses[f].reshape(-1))
        d = np.ascontiguousarray(s.dist[f].reshape(-1))
        o.update(d, Tf, Kc)
        L.ref_tsdf_update(O.ptr(ref), R, O.ptr(org), O.ptr(dm), W, H, p.min_dist, p.max_dist, O.ptr(Tf), O.ptr(Kc),
                          O.ptr(d))
        assert np.array_equal(bits(ref), bits(o.grid)), f
    for f in range(3):
        Tf = np.ascontiguousarray(poses[f].reshape(-1))
        xyz = o.raycast(Tf, Kc)
        xr = np.zeros_like(xyz)
        L.ref_tsdf_raycast(O.ptr(ref), R, O.ptr(org), O.ptr(dm), W, H, p.min_dist, p.max_dist, O.ptr(Tf), O.ptr(Kc),
                           1, O.ptr(xr))
        assert np.array_equal(bits(xyz), bits(xr)), f
        if f != 1:
            # the straight-ahead column and row hit the wall (their rays have a zero component)
            img = xyz.reshape(H, W, 4)
            assert img[3:-3, 80, 3].all() and img[60, 3:-3, 3].all(), f
