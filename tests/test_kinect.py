"""Kinect pre-processing (tracker/multicore/multicore.cpp): disparity -> depth
at full and half resolution, RGB -> gray, undistortion of a gray image.

CPU: the oracle (oracle/oracle_kinect.c) equals the reference's own routines
(built for the host by oracle/build_ref.py) bit for bit.  GPU: the kernels
(recon_kinect_*) equal the oracle bit for bit."""
import numpy as np
import pytest

import oracle_lib as O
import ref_lib as RL
from recon_gb300 import synth

needs_ref = pytest.mark.skipif(not RL.available(), reason="oracle/_ref not built (reference tree absent)")
SIZES = [(640, 480), (322, 246)]


def inputs(W, H, seed=1):
    rng = np.random.default_rng(seed)
    cal = synth.make_calibration(W, H, distortion=True)
    c0, c1 = np.float32(cal.calib[61]), np.float32(cal.calib[42])
    disp = rng.integers(280, 1040, (H, W)).astype(np.uint16)
    disp[rng.random((H, W)) < 0.05] = 2047
    disp[rng.random((H, W)) < 0.01] = 1200  # beyond max_dist
    rgb = rng.integers(0, 256, (H, W, 3)).astype(np.uint8)
    gray = rng.integers(0, 256, (H, W)).astype(np.uint8)
    K = np.ascontiguousarray(cal.calib[0:9], np.float32)
    iK = np.ascontiguousarray(cal.calib[9:18], np.float32)
    kc = np.ascontiguousarray(cal.calib[18:23], np.float32)
    return cal, c0, c1, disp, rgb, gray, K, iK, kc


def oracle_all(W, H, seed=1):
    cal, c0, c1, disp, rgb, gray, K, iK, kc = inputs(W, H, seed)
    L = O.lib()
    out = {}
    for xo, yo in [(0.0, 0.0), (-4.0, -3.0)]:
        z = np.zeros((H, W), np.float32)
        L.orc_kinect_d2z(O.ptr(disp), W, H, c0, c1, cal.min_dist, cal.max_dist, xo, yo, O.ptr(z))
        out[("z", xo)] = z
        zl = np.zeros((H // 2, W // 2), np.float32)
        L.orc_kinect_d2z_low(O.ptr(disp), W // 2, H // 2, c0, c1, cal.min_dist, cal.max_dist, xo, yo, O.ptr(zl))
        out[("zl", xo)] = zl
    g = np.zeros((H, W), np.uint8)
    L.orc_kinect_rgb2gray(O.ptr(rgb), W, H, O.ptr(g))
    out["gray"] = g
    u = np.zeros((H, W), np.uint8)
    L.orc_kinect_undistort(O.ptr(gray), W, H, O.ptr(K), O.ptr(iK), O.ptr(kc), O.ptr(u))
    out["undistort"] = u
    return out


@needs_ref
@pytest.mark.parametrize("W,H", SIZES)
def test_oracle_matches_reference_routines(W, H):
    cal, c0, c1, disp, rgb, gray, K, iK, kc = inputs(W, H)
    o = oracle_all(W, H)
    R = RL.lib()
    for xo, yo in [(0.0, 0.0), (-4.0, -3.0)]:
        z = np.zeros((H, W), np.float32)
        R.ref_d2Z(O.ptr(disp), W, H, c0, c1, cal.min_dist, cal.max_dist, xo, yo, O.ptr(z))
        assert np.array_equal(z.view(np.uint32), o[("z", xo)].view(np.uint32)), xo
        zl = np.zeros((H // 2, W // 2), np.float32)
        R.ref_d2ZLow(O.ptr(disp), W // 2, H // 2, c0, c1, cal.min_dist, cal.max_dist, xo, yo, O.ptr(zl))
        assert np.array_equal(zl.view(np.uint32), o[("zl", xo)].view(np.uint32)), xo
    assert (o[("z", 0.0)] > 0).mean() > 0.8 and (o[("zl", 0.0)] > 0).mean() > 0.6
    # the shift leaves the first 4 columns and 3 rows without depth
    assert not o[("z", -4.0)][:, :4].any() and not o[("z", -4.0)][:3].any()
    g = np.zeros((H, W), np.uint8)
    R.ref_convert2Gray(O.ptr(rgb), W, H, O.ptr(g))
    assert np.array_equal(g, o["gray"])
    u = np.zeros((H, W), np.uint8)
    for calls in (2, 3):  # the lookup form every call after the first uses
        R.ref_undistort(O.ptr(gray), W, H, O.ptr(K), O.ptr(iK), O.ptr(kc), calls, O.ptr(u))
        assert np.array_equal(u, o["undistort"]), calls
    # the first call (direct mapping) differs at most by rounding of the offsets
    R.ref_undistort(O.ptr(gray), W, H, O.ptr(K), O.ptr(iK), O.ptr(kc), 1, O.ptr(u))
    assert np.mean(u != o["undistort"]) < 1e-3


@pytest.mark.gpu
@pytest.mark.parametrize("W,H", SIZES)
def test_kinect_kernels_match_oracle(W, H):
    import torch
    import recon_gb300 as rg
    cal, c0, c1, disp, rgb, gray, K, iK, kc = inputs(W, H)
    o = oracle_all(W, H)
    d = torch.from_numpy(disp.view(np.int16)).cuda()
    for xo, yo in [(0.0, 0.0), (-4.0, -3.0)]:
        z = rg.kinect_disparity_to_depth(d, float(c0), float(c1), cal.min_dist, cal.max_dist, xo, yo).cpu().numpy()
        assert np.array_equal(z.view(np.uint32), o[("z", xo)].view(np.uint32)), xo
        zl = rg.kinect_disparity_to_depth(d, float(c0), float(c1), cal.min_dist, cal.max_dist, xo, yo,
                                          half_resolution=True).cpu().numpy()
        assert np.array_equal(zl.view(np.uint32), o[("zl", xo)].view(np.uint32)), xo
    g = rg.kinect_rgb_to_gray(torch.from_numpy(rgb).cuda()).cpu().numpy()
    assert np.array_equal(g, o["gray"])
    u = rg.kinect_undistort_gray(torch.from_numpy(gray).cuda(), K, iK, kc).cpu().numpy()
    assert np.array_equal(u, o["undistort"])
