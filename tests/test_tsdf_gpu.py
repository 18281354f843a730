"""The reconstruction stream on the GPU (recon_tsdf_*) against the CPU oracle:
bit-identical grids after every update, ray-cast points, shading, normals,
resampling and distance maps; the brick bytes never hide a negative voxel;
argument errors are reported, not run."""
import numpy as np
import pytest

import oracle_lib as O
from scenes import depth_sequence

pytestmark = pytest.mark.gpu

CUBES = {
    "reference": (O.TSDF_ORIGIN, O.TSDF_DIM),
    "room": ((0.0, 150.0, -2350.0), (1750.0, 1750.0, 1750.0)),
}


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def _flags_cover_negatives(grid, flags, R):
    g = grid.reshape(R, R, R, 2)[..., 0]
    neg = g < 0
    b = R // 8
    need = neg.reshape(b, 8, b, 8, b, 8).any(axis=(1, 3, 5)).reshape(-1)
    return bool(np.all(flags[need] != 0))


@pytest.mark.parametrize("W,H,R,cube,noise", [
    (160, 120, 64, "reference", 0.001),
    (160, 120, 64, "room", 0.0),
    (320, 240, 128, "room", 0.001),
    (200, 150, 40, "room", 0.0),  # R not a multiple of 32, image not a multiple of 16
])
def test_tsdf_matches_oracle(W, H, R, cube, noise):
    import recon_gb300 as rg
    s = depth_sequence(W, H, 5, seed=5, noise=noise)
    origin, dim = CUBES[cube]
    op = O.tsdf_params(R, W, H, origin=origin, dim=dim)
    o = O.OracleTSDF(op)
    v = rg.TSDF(rg.tsdf_params(R, W, H, cube_origin=origin, cube_dim=dim))
    assert np.array_equal(bits(v.get("tsdf")), bits(o.grid))
    v.enable_counting(True)
    for f in range(5):
        v.set_dist_map(s.dist[f])
        v.update(s.poses[f], s.K)
        o.update(s.dist[f], s.poses[f], s.K)
        g = v.get("tsdf")
        assert np.array_equal(bits(g), bits(o.grid)), f
        assert _flags_cover_negatives(g, v.get("flags"), R)
        c = v.counts()
        assert c[0] >= c[1] >= c[2] >= 0 and c[1] > 0
    for f in (0, 4):
        for cubic in (False, True):
            v.raycast(s.poses[f], s.K, cubic_filter=cubic)
            xyz = o.raycast(s.poses[f], s.K, filtering=cubic)
            assert np.array_equal(bits(v.get("xyz")), bits(xyz)), (f, cubic)
        sh, nr = o.shade(xyz)
        assert np.array_equal(bits(v.get("shaded")), bits(sh))
        assert np.array_equal(bits(v.get("normal")), bits(nr))
    assert (xyz[3::4] > 0).mean() > 0.005
    # resampling into a second grid of the same parameters
    v2 = rg.TSDF(rg.tsdf_params(R, W, H, cube_origin=origin, cube_dim=dim))
    v2.resample_from(v, s.poses[2])
    rs = o.resampled(s.poses[2])
    g2 = v2.get("tsdf")
    assert np.array_equal(bits(g2), bits(rs))
    assert _flags_cover_negatives(g2, v2.get("flags"), R)
    v2.close()
    v.close()


def test_tsdf_measurements_and_device_inputs():
    """uint16 depth and the float4 RGB-D frame give the oracle's distance map;
    device (torch) inputs equal host inputs; a replaced grid rebuilds the brick
    bytes; reset restores (1, 0)."""
    import torch
    import recon_gb300 as rg
    from test_tsdf_oracle import rgbd_frame
    W, H, R = 160, 120, 64
    s = depth_sequence(W, H, 3, seed=9, noise=0.001)
    origin, dim = CUBES["room"]
    v = rg.TSDF(rg.tsdf_params(R, W, H, cube_origin=origin, cube_dim=dim))
    v.set_dist_depth16(s.depth[0])
    assert np.array_equal(bits(v.get("dist")), bits(s.dist[0].reshape(-1)))
    v.set_dist_depth16(torch.from_numpy(np.ascontiguousarray(s.depth[1]).view(np.int16)).cuda())  # same bytes
    assert np.array_equal(bits(v.get("dist")), bits(s.dist[1].reshape(-1)))
    rgbd = rgbd_frame(s.dist[2], 400.0, 4500.0)
    d_o = np.zeros(W * H, np.float32)
    O.lib().orc_tsdf_dist_from_rgbd(O.ptr(rgbd), W, H, 400.0, 4500.0, O.ptr(d_o))
    v.set_dist_rgbd_float4(rgbd)
    assert np.array_equal(bits(v.get("dist")), bits(d_o))
    v.set_dist_rgbd_float4(torch.from_numpy(rgbd).cuda())
    assert np.array_equal(bits(v.get("dist")), bits(d_o))
    # device distance map, then update from it
    o = O.OracleTSDF(O.tsdf_params(R, W, H, origin=origin, dim=dim))
    v.reset()
    v.set_dist_map(torch.from_numpy(s.dist[0]).cuda())
    v.update(s.poses[0], s.K)
    o.update(s.dist[0], s.poses[0], s.K)
    assert np.array_equal(bits(v.get("tsdf")), bits(o.grid))
    # a grid given from outside: the brick bytes are rebuilt from it
    g = o.grid.copy()
    g[0::2][12345] = -0.5
    v.set_grid(torch.from_numpy(g).cuda())
    assert np.array_equal(bits(v.get("tsdf")), bits(g))
    assert _flags_cover_negatives(g, v.get("flags"), R)
    v.raycast(s.poses[0], s.K)
    o.grid[:] = g
    assert np.array_equal(bits(v.get("xyz")), bits(o.raycast(s.poses[0], s.K)))
    v.reset()
    g = v.get("tsdf")
    assert np.all(g[0::2] == 1.0) and np.all(g[1::2] == 0.0) and not v.get("flags").any()
    v.close()


def test_tsdf_argument_errors():
    import recon_gb300 as rg
    with pytest.raises(rg.ReconError):
        rg.TSDF(rg.tsdf_params(60, 160, 120))  # not a multiple of 8
    with pytest.raises(rg.ReconError):
        rg.TSDF(rg.tsdf_params(64, 4, 120))
    v = rg.TSDF(rg.tsdf_params(64, 160, 120))
    K = np.array([0.5, 0, 0.5, 0, 0.6, 0.5, 0, 0, 1], np.float32)
    bad = np.eye(4, dtype=np.float32)
    bad[0, 3] = np.nan
    with pytest.raises(rg.ReconError):
        v.update(bad, K)
    with pytest.raises(rg.ReconError):
        v.raycast(np.eye(4, dtype=np.float32), np.zeros(9, np.float32))
    other = rg.TSDF(rg.tsdf_params(32, 160, 120))
    with pytest.raises(rg.ReconError):
        other.resample_from(v, np.eye(4, dtype=np.float32))
    # the grid is still usable after the rejected calls
    v.update(np.eye(4, dtype=np.float32), K)
    assert np.all(v.get("tsdf")[0::2] == 1.0)
    other.close()
    v.close()


def test_tsdf_traversal_edge_cases_match_oracle():
    """A camera inside the grid, axis-aligned poses and rays with an exactly
    zero direction component (the traversal's FLT_MAX inverse) on the GPU."""
    import recon_gb300 as rg
    from test_tsdf_oracle import edge_case_setup
    s, K, poses, p = edge_case_setup()
    o = O.OracleTSDF(p)
    v = rg.TSDF(rg.tsdf_params(p.R, p.W, p.H, cube_origin=tuple(p.origin), cube_dim=tuple(p.dim)))
    for f in range(3):
        v.set_dist_map(s.dist[f])
        v.update(poses[f], K)
        o.update(s.dist[f], poses[f], K)
    assert np.array_equal(bits(v.get("tsdf")), bits(o.grid))
    for f in range(3):
        v.raycast(poses[f], K)
        assert np.array_equal(bits(v.get("xyz")), bits(o.raycast(poses[f], K))), f
    v.close()
