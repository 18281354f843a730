"""Kinect pre-processing.  The host routines of tracker/multicore/multicore.cpp:
disparity -> depth at full and half resolution, RGB -> gray, undistortion of
a gray image.  The GPU capture path (d2z.cu, rgb2gray.cu, undistort.cu, as
capture/VideoPreProcessorGPU.cpp and reconstruct/TrackFrame.cpp call it):
disparity as float, normalised half-resolution depth from 16-bit or float
disparity, RGB -> float RGB, RGB / float RGB -> float gray, undistortion of
an RGB image into float RGB.

CPU: the oracle (oracle/oracle_kinect.c) equals the reference's own code
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
    disp[rng.random((H, W)) < 0.01] = 1200  # past the pole of 1 / (c0 + c1 d): a negative denominator
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


def capture_inputs(W, H, seed=2):
    cal, c0, c1, disp, rgb, gray, K, iK, kc = inputs(W, H, seed)
    disp[100:110, 100:110] = 1040  # a patch beyond max_dist (about 7 m)
    calib = np.zeros(96, np.float32)
    calib[:96] = cal.calib[:96]
    calib[61], calib[42], calib[62], calib[63] = c0, c1, cal.min_dist, cal.max_dist
    return cal, c0, c1, disp, rgb, K, iK, kc, calib


def oracle_capture(W, H, seed=2):
    cal, c0, c1, disp, rgb, K, iK, kc, calib = capture_inputs(W, H, seed)
    L = O.lib()
    n = W * H
    out = {}
    u = np.zeros((H, W), np.float32)
    L.orc_kinect_disparity_to_float(O.ptr(disp), n, O.ptr(u))
    out["disp_f"] = u
    for xo, yo in [(0.0, 0.0), (-4.0, -3.0)]:
        z = np.zeros((H // 2, W // 2), np.float32)
        L.orc_kinect_depth_normalized(O.ptr(disp), None, W, H, c0, c1, cal.min_dist, cal.max_dist, xo, yo, O.ptr(z))
        out[("zn", xo)] = z
        zf = np.zeros((H // 2, W // 2), np.float32)
        L.orc_kinect_depth_normalized(None, O.ptr(u), W, H, c0, c1, cal.min_dist, cal.max_dist, xo, yo, O.ptr(zf))
        out[("zn_hdr", xo)] = zf
    hdr = np.zeros((H, W, 3), np.float32)
    L.orc_kinect_rgb_to_hdr(O.ptr(rgb), n, O.ptr(hdr))
    out["rgb_hdr"] = hdr
    g = np.zeros((H, W), np.float32)
    L.orc_kinect_rgb_to_gray_hdr(O.ptr(rgb), n, O.ptr(g))
    out["gray_hdr_u8"] = g
    g2 = np.zeros((H, W), np.float32)
    L.orc_kinect_rgb_hdr_to_gray(O.ptr(hdr), n, O.ptr(g2))
    out["gray_hdr_f"] = g2
    ur = np.zeros((H, W, 3), np.float32)
    L.orc_kinect_undistort_rgb_hdr(O.ptr(rgb), W, H, O.ptr(K), O.ptr(iK), O.ptr(kc), O.ptr(ur))
    out["undistort_rgb"] = ur
    return out


def _same(a, b):
    return np.array_equal(np.asarray(a).view(np.uint32), np.asarray(b).view(np.uint32))


@needs_ref
@pytest.mark.parametrize("W,H", [(640, 480), (320, 240)])
def test_capture_path_oracle_matches_reference_kernels(W, H):
    cal, c0, c1, disp, rgb, K, iK, kc, calib = capture_inputs(W, H)
    o = oracle_capture(W, H)
    R = RL.lib()
    u = np.zeros((H, W), np.float32)
    R.ref_undistortDisparity(O.ptr(disp), O.ptr(u), W, H, O.ptr(calib))
    assert _same(u, o["disp_f"])
    assert (u == 65535).any() and (u < 2047).mean() > 0.9
    for xo, yo in [(0.0, 0.0), (-4.0, -3.0)]:
        for key, fn, src in (("zn", R.ref_d2ZLowGpu, disp), ("zn_hdr", R.ref_d2ZLowHdrGpu, u)):
            z = np.zeros((H // 2, W // 2), np.float32)
            fn(O.ptr(src), O.ptr(z), W, H, O.ptr(calib), xo, yo)
            want = o[(key, xo)]
            if xo == 0.0:
                assert _same(z, want), key
            else:
                # compiled for the host, 2x - 4 < 0 wraps to an out-of-range
                # index (no depth); on the GPU it saturates to column 0, which
                # the oracle follows: the two differ only in columns 0-1 and
                # rows 0-1
                assert _same(z[2:, 2:], want[2:, 2:]), key
                assert not z[:2].any() and not z[:, :2].any()
                assert want[:2].any() and want[:, :2].any()
            # depth inside [min_dist, max_dist] maps to [0, 1], outside it to
            # (0 - min_dist) / (max_dist - min_dist)
            v = want[want != 0]
            low = np.float32(-cal.min_dist / (cal.max_dist - cal.min_dist))
            assert v.size > 0.6 * want.size and np.all(((v >= 0) & (v <= 1)) | np.isclose(v, low))
            assert np.isclose(want[52:54, 52:54], low).all()
    hdr = np.zeros((H, W, 3), np.float32)
    R.ref_convertHdrRGB(O.ptr(rgb), O.ptr(hdr), W, H)
    assert _same(hdr, o["rgb_hdr"])
    g = np.zeros((H, W), np.float32)
    R.ref_rgb2GrayHdr(O.ptr(rgb), O.ptr(g), W, H)
    assert _same(g, o["gray_hdr_u8"])
    R.ref_rgbF2GrayHdr(O.ptr(hdr), O.ptr(g), W, H)
    assert _same(g, o["gray_hdr_f"])
    ur = np.zeros((H, W, 3), np.float32)
    R.ref_undistortHdrRGB(O.ptr(rgb), O.ptr(ur), W, H, O.ptr(calib))
    assert _same(ur, o["undistort_rgb"])
    assert (ur == 0).all(axis=2).mean() < 0.1


@pytest.mark.gpu
@pytest.mark.parametrize("W,H", [(640, 480), (322, 246)])
def test_capture_path_kernels_match_oracle(W, H):
    import torch
    import recon_gb300 as rg
    cal, c0, c1, disp, rgb, K, iK, kc, calib = capture_inputs(W, H)
    o = oracle_capture(W, H)
    d = torch.from_numpy(disp.view(np.int16)).cuda()
    u = rg.kinect_disparity_to_float(d)
    assert _same(u.cpu().numpy(), o["disp_f"])
    for xo, yo in [(0.0, 0.0), (-4.0, -3.0)]:
        z = rg.kinect_depth_normalized(d, float(c0), float(c1), cal.min_dist, cal.max_dist, xo, yo)
        assert _same(z.cpu().numpy(), o[("zn", xo)]), xo
        zf = rg.kinect_depth_normalized(u, float(c0), float(c1), cal.min_dist, cal.max_dist, xo, yo)
        assert _same(zf.cpu().numpy(), o[("zn_hdr", xo)]), xo
    r = torch.from_numpy(rgb).cuda()
    hdr = rg.kinect_rgb_to_hdr(r)
    assert _same(hdr.cpu().numpy(), o["rgb_hdr"])
    assert _same(rg.kinect_rgb_to_gray_hdr(r).cpu().numpy(), o["gray_hdr_u8"])
    assert _same(rg.kinect_rgb_to_gray_hdr(hdr).cpu().numpy(), o["gray_hdr_f"])
    assert _same(rg.kinect_undistort_rgb_hdr(r, K, iK, kc).cpu().numpy(), o["undistort_rgb"])


@pytest.mark.gpu
def test_capture_path_argument_errors():
    import torch
    import recon_gb300 as rg
    d = torch.zeros((4, 6), dtype=torch.int16, device="cuda")
    L = rg.lib()
    z = torch.zeros((2, 3), dtype=torch.float32, device="cuda")
    # both or neither disparity input, odd size
    assert L.recon_kinect_depth_normalized(None, None, 6, 4, 1.0, 1.0, 0.0, 1.0, 0.0, 0.0, z.data_ptr(), None) != 0
    assert L.recon_kinect_depth_normalized(d.data_ptr(), z.data_ptr(), 6, 4, 1.0, 1.0, 0.0, 1.0, 0.0, 0.0,
                                           z.data_ptr(), None) != 0
    assert L.recon_kinect_depth_normalized(d.data_ptr(), None, 5, 4, 1.0, 1.0, 0.0, 1.0, 0.0, 0.0, z.data_ptr(),
                                           None) != 0
    assert L.recon_kinect_rgb_to_gray_hdr(None, None, 6, 4, z.data_ptr(), None) != 0
