"""Pins the CPU oracle to the reference's own kernel code.

oracle/_ref/libreconref.so holds the reference's one-thread-per-element kernels
(warp.cu, histogram64.cu, d2z.cu, rgb2gray.cu, downSample2Cuda.cu) and its CPU
expm (expm.c) compiled for the host from the reference tree.  Each stage of the
oracle must reproduce them bit for bit on the same inputs, except where a
difference is deliberate and documented (reduction order, Student-t sum,
out-of-image taps at the coarsest level, the SE(3) exponential's arithmetic).
"""
import ctypes

import numpy as np
import pytest

import oracle_lib as O
import ref_lib as R
from pose_book import apply_increment_ref_order
from recon_gb300 import synth

pytestmark = pytest.mark.skipif(not R.available(), reason="reference tree not built into oracle/_ref")

p = O.ptr


@pytest.fixture(scope="module", params=[(320, 240, 3), (640, 480, 4)], ids=["320x240", "640x480"])
def frame_pair(request):
    W, H, L = request.param
    cal = synth.make_calibration(W, H, distortion=(L == 4))
    sc = synth.make_scene(11)
    Tref = np.eye(4)
    Tcur = Tref @ synth.offset_pose(4, 2.0, 20.0)
    g0, d0 = O.render_pair(sc, synth.camera_struct(cal, "L", Tref), synth.camera_struct(cal, "R", Tref), frame=0)
    g1, d1 = O.render_pair(sc, synth.camera_struct(cal, "L", Tcur), synth.camera_struct(cal, "R", Tcur), frame=1)
    return dict(W=W, H=H, L=L, cal=cal, g0=g0, d0=d0, g1=g1, d1=d1,
                T=synth.relative_pose(Tref, Tcur).astype(np.float32))


def _pyr(gray_u8, L):
    W = gray_u8.shape[1]
    H = gray_u8.shape[0]
    lv = [(gray_u8.astype(np.float32) / np.float32(255.0)).astype(np.float32).reshape(-1)]
    for l in range(1, L):
        lo = np.zeros((H >> l) * (W >> l), np.float32)
        O.lib().orc_downsample2(p(lv[-1]), W >> l, H >> l, p(lo))
        lv.append(lo)
    return lv


def test_gray_pyramid_matches_reference(frame_pair):
    fp = frame_pair
    lv = _pyr(fp["g0"], fp["L"])
    for l in range(1, fp["L"]):
        ref = np.zeros_like(lv[l])
        R.lib().ref_fastDownSampleHdr(p(lv[l - 1]), fp["W"] >> l, fp["H"] >> l, p(ref))
        assert np.array_equal(ref.view(np.uint32), lv[l].view(np.uint32))


def _reference_prep(fp):
    """Oracle and reference vertex records + selection for the reference frame."""
    W, H, L, calib = fp["W"], fp["H"], fp["L"], fp["cal"].calib
    z = np.zeros(W * H, np.float32)
    d0 = fp["d0"].reshape(-1).copy()
    O.lib().orc_convert_depth(p(d0), W * H, p(z))
    xyz_o = np.zeros(4 * W * H, np.float32)
    xyz_r = np.zeros(4 * W * H, np.float32)
    O.lib().orc_zmap_to_xyz(p(z), W, H, p(calib), p(xyz_o))
    R.lib().ref_convertZMapToXYZ(p(z), p(xyz_r), p(calib), W, H)
    lv = _pyr(fp["g0"], L)
    vd_o = np.zeros(24 * W * H, np.float32)
    vd_r = np.zeros(24 * W * H, np.float32)
    O.lib().orc_xyz2cloud(p(xyz_o), W, H, p(calib), p(lv[0]), p(vd_o))
    R.lib().ref_xyz2Cloud(p(xyz_r), W, H, p(calib), p(vd_r), p(lv[0]))
    return z, xyz_o, xyz_r, lv, vd_o, vd_r


def test_zmap_and_vertex_records_match_reference(frame_pair):
    z, xyz_o, xyz_r, lv, vd_o, vd_r = _reference_prep(frame_pair)
    assert np.array_equal(xyz_o.view(np.uint32), xyz_r.view(np.uint32))
    rec_o = vd_o.reshape(-1, 24)[:, :15]
    rec_r = vd_r.reshape(-1, 24)[:, :15]
    assert np.array_equal(rec_o.view(np.uint32), rec_r.view(np.uint32))


def _select(fp, vd):
    W, H = fp["W"], fp["H"]
    grad = np.ascontiguousarray(vd.reshape(-1, 24)[:, 13])
    hist = np.zeros(256, np.int32)
    O.lib().orc_grad_histogram(p(grad), W * H, 256, p(hist))
    idx = np.zeros(8192, np.int32)
    O.lib().orc_filter_indices(p(grad), W * H, p(hist), 256, 8192, p(idx))
    return idx


def test_attributes_and_jacobians_match_reference(frame_pair):
    fp = frame_pair
    W, H, L, calib = fp["W"], fp["H"], fp["L"], fp["cal"].calib
    z, xyz_o, xyz_r, lv, vd_o, vd_r = _reference_prep(fp)
    idx = _select(fp, vd_o)
    # the reference reads up to one row/column outside the coarsest 4-level image:
    # give it padded copies so that its reads stay in allocated memory
    pad = 4 * (W >> 1)
    padded = []
    for l in range(L):
        buf = np.full(lv[l].size + 2 * pad, -1.0, np.float32)
        buf[pad:pad + lv[l].size] = lv[l]
        padded.append(buf)
    ptrs_r = [ctypes.c_void_p(b.ctypes.data + 4 * pad) for b in padded] + [ctypes.c_void_p(0)] * (4 - L)
    O.lib().orc_add_vertex_attributes(p(idx), 8192, p(vd_o), W, H, p(calib), O.ptrs(lv), L)
    R.lib().ref_addVertexAttributes(p(idx), 8192, p(vd_r), W, H, p(calib), *ptrs_r, L)
    ro = vd_o.reshape(-1, 24)[idx]
    rr = vd_r.reshape(-1, 24)[idx]
    slots = list(range(15, 15 + 3 * (L - 1)))
    if L == 3:
        assert np.array_equal(ro[:, slots].view(np.uint32), rr[:, slots].view(np.uint32))
    else:
        # coarsest level: compare the points whose 5-tap stencil lies inside the image
        px = ro[:, 6]
        py = ro[:, 7]
        l3x = ((px * 0.5 - 0.25) * 0.5 - 0.25) * 0.5 - 0.25
        l3y = ((py * 0.5 - 0.25) * 0.5 - 0.25) * 0.5 - 0.25
        inside = (l3x >= 1) & (l3y >= 1) & (l3x < (W >> 3) - 2) & (l3y < (H >> 3) - 2)
        assert inside.mean() > 0.9
        assert np.array_equal(ro[:, 15:21].view(np.uint32), rr[:, 15:21].view(np.uint32))
        assert np.array_equal(ro[inside][:, 21:24].view(np.uint32), rr[inside][:, 21:24].view(np.uint32))
        vd_r.reshape(-1, 24)[idx, 21:24] = ro[:, 21:24]  # continue with identical inputs
    Jo = [np.zeros(6 * 8192, np.float32) for _ in range(4)]
    Jr = [np.zeros(6 * 8192, np.float32) for _ in range(4)]
    O.lib().orc_precompute_jacobian(p(idx), 8192, p(vd_o), p(calib), 1e-3, L, O.ptrs(Jo))
    R.lib().ref_precomputeJacobian4(p(idx), 8192, p(vd_o), p(calib), *[p(j) for j in Jr], 1e-3)
    for l in range(L):
        assert np.array_equal(Jo[l].view(np.uint32), Jr[l].view(np.uint32)), f"level {l}"


def test_residual_weights_match_reference(frame_pair):
    fp = frame_pair
    W, H, L, calib = fp["W"], fp["H"], fp["L"], fp["cal"].calib
    z, xyz_o, xyz_r, lv, vd_o, vd_r = _reference_prep(fp)
    idx = _select(fp, vd_o)
    O.lib().orc_add_vertex_attributes(p(idx), 8192, p(vd_o), W, H, p(calib), O.ptrs(lv), L)
    rec = vd_o.reshape(-1, 24)[idx]
    sel_xyz = np.ascontiguousarray(rec[:, :3].T).reshape(-1)
    zc = np.zeros(W * H, np.float32)
    d1 = fp["d1"].reshape(-1).copy()
    O.lib().orc_convert_depth(p(d1), W * H, p(zc))
    cur = _pyr(fp["g1"], L)
    # a pose between identity and the truth: residuals of mixed sign, some out of view
    T = np.ascontiguousarray((0.5 * (np.eye(4) + fp["T"])).astype(np.float32)).reshape(-1)
    for l in range(L):
        I = np.ascontiguousarray(rec[:, [14, 17, 20, 23][l]])
        ro, zo = np.zeros(8192, np.float32), np.zeros(8192, np.float32)
        rr, zr = np.zeros(8192, np.float32), np.zeros(8192, np.float32)
        O.lib().orc_interpolate_residual(8192, p(sel_xyz), p(I), p(T), p(calib), l, p(cur[l]), W >> l, H >> l,
                                         p(zc), W, H, p(ro), p(zo))
        R.lib().ref_interpolateResidual2(p(idx), 8192, p(vd_o), p(T), p(calib), l, p(cur[l]), W >> l, H >> l,
                                         p(zc), W, H, p(rr), p(zr))
        assert np.array_equal(ro.view(np.uint32), rr.view(np.uint32)), f"residual level {l}"
        assert np.array_equal(zo.view(np.uint32), zr.view(np.uint32)), f"zweight level {l}"
        ho, wo, rwo = np.zeros(64, np.int32), np.zeros(8192, np.float32), np.zeros(8192, np.float32)
        hr, wr, rwr = np.zeros(64, np.int32), np.zeros(8192, np.float32), np.zeros(8192, np.float32)
        mo = O.lib().orc_generate_weights(p(ro), p(zo), 8192, 64, p(ho), p(wo), p(rwo))
        mr = R.lib().ref_generateWeights64(p(rr), 8192, p(wr), p(zr), p(rwr), p(hr))
        assert mo == mr
        assert np.array_equal(ho, hr)
        assert np.array_equal(wo.view(np.uint32), wr.view(np.uint32))
        assert np.array_equal(rwo.view(np.uint32), rwr.view(np.uint32))


def test_icp_stages_match_reference(frame_pair):
    fp = frame_pair
    W, H, L, calib = fp["W"], fp["H"], fp["L"], fp["cal"].calib
    lib, ref = O.lib(), R.lib()
    zr = np.zeros(W * H, np.float32)
    zc = np.zeros(W * H, np.float32)
    d0, d1 = fp["d0"].reshape(-1).copy(), fp["d1"].reshape(-1).copy()
    lib.orc_convert_depth(p(d0), W * H, p(zr))
    lib.orc_convert_depth(p(d1), W * H, p(zc))
    ro6, rm_o = np.zeros(6 * W * H, np.float32), np.zeros(W * H, np.int32)
    rr6, rm_r = np.zeros(6 * W * H, np.float32), np.zeros(W * H, np.int32)
    lib.orc_zmap_to_xyz6(p(zr), W, H, p(calib), p(ro6), p(rm_o))
    ref.ref_convertZMapToXYZ6(p(zr), p(rr6), p(rm_r), p(calib), W, H)
    lib.orc_compute_normals6(p(ro6), p(rm_o), W, H)
    ref.ref_computeNormals(p(rr6), p(rm_r), W, H)
    assert np.array_equal(rm_o, rm_r)
    assert np.array_equal(ro6.view(np.uint32), rr6.view(np.uint32))
    co6, cm_o = np.zeros(6 * W * H, np.float32), np.zeros(W * H, np.int32)
    cr6, cm_r = np.zeros(6 * W * H, np.float32), np.zeros(W * H, np.int32)
    lib.orc_gen_cloud6(p(zc), W, H, p(calib), p(co6), p(cm_o))
    ref.ref_genPointsCloud6(p(zc), W, H, p(calib), p(cr6), p(cm_r))
    assert np.array_equal(cm_o, cm_r) and np.array_equal(co6.view(np.uint32), cr6.view(np.uint32))
    refs, curs = [(ro6, rm_o)], [(co6, cm_o)]
    for l in range(1, L):
        w, h = W >> l, H >> l
        for pyr in (refs, curs):
            src, msrc = pyr[-1]
            d_o, m_o = np.zeros(6 * w * h, np.float32), np.zeros(w * h, np.int32)
            d_r, m_r = np.zeros(6 * w * h, np.float32), np.zeros(w * h, np.int32)
            lib.orc_downsample_cloud6(p(src), p(msrc), w, h, p(d_o), p(m_o))
            ref.ref_downSampleCloud6(p(src), p(msrc), p(d_r), p(m_r), w, h)
            assert np.array_equal(m_o, m_r)
            assert np.array_equal(d_o.view(np.uint32), d_r.view(np.uint32))
            pyr.append((d_o, m_o))
    T = np.ascontiguousarray((0.5 * (np.eye(4) + fp["T"])).astype(np.float32)).reshape(-1)
    for l in range(L):
        w, h = W >> l, H >> l
        res_o, msk_o = np.zeros(w * h, np.float32), np.zeros(w * h, np.int32)
        res_r, msk_r = np.zeros(w * h, np.float32), np.zeros(w * h, np.int32)
        lib.orc_icp_residual_mask(p(refs[l][0]), p(refs[l][1]), w, h, p(T), p(calib), p(curs[l][0]), p(curs[l][1]),
                                  l, p(res_o), p(msk_o))
        ref.ref_icpResidualMask2(p(refs[l][0]), p(refs[l][1]), w, h, p(T), p(calib), p(curs[l][0]), p(curs[l][1]),
                                 l, p(res_r), p(msk_r))
        assert np.array_equal(msk_o, msk_r), f"mask level {l}"
        on = msk_o > 0
        assert np.array_equal(res_o[on].view(np.uint32), res_r[on].view(np.uint32))
        sel = np.zeros(w * h, np.int32)
        n = lib.orc_compact(p(msk_o), w * h, p(sel))
        assert n == int(on.sum()) and np.array_equal(sel[:n], np.flatnonzero(on))
        r = np.ascontiguousarray(res_o[sel[:n]])
        r2 = (r * r).astype(np.float32)
        w_o = np.zeros(n, np.float32)
        w_r = np.zeros(n, np.float32)
        lib.orc_student_t(p(r2), n, p(w_o))
        ref.ref_studentT(p(r2), n, p(w_r))
        # exact int64 sum vs the reference's float tree: equal unless partial sums pass 2^24
        np.testing.assert_allclose(w_o, w_r, rtol=2e-6, atol=0)
        npad = ((n + 1023) // 1024) * 1024
        jo, jr = np.zeros(6 * npad, np.float32), np.zeros(6 * npad, np.float32)
        eo, er = np.zeros(npad, np.float32), np.zeros(npad, np.float32)
        lib.orc_icp_residual_jacobian(p(refs[l][0]), p(sel), n, w, h, l, p(T), p(calib), p(curs[l][0]),
                                      p(curs[l][1]), npad, p(eo), p(jo), p(w_o), 1e-3)
        ref.ref_icpResidual2(p(refs[l][0]), p(sel), n, w, h, l, p(T), p(calib), p(curs[l][0]), p(curs[l][1]), npad,
                             p(er), p(jr), p(w_o), 1e-3)
        assert np.array_equal(eo.view(np.uint32), er.view(np.uint32)), f"icp residual level {l}"
        assert np.array_equal(jo.view(np.uint32), jr.view(np.uint32)), f"icp jacobian level {l}"
        # the tracker's form over the pixel grid (fused multiply-adds in the
        # continuous terms): the same pixels are correspondences, and every
        # residual and Jacobian entry is within 1e-5 of the reference's,
        # relative to the largest entry of its column at the level
        wpx = np.zeros(w * h, np.float32)
        wpx[sel[:n]] = w_o
        gpad = ((w * h + 1023) // 1024) * 1024
        jg, eg = np.zeros(6 * gpad, np.float32), np.zeros(gpad, np.float32)
        lib.orc_icp_residual_jacobian_grid(p(refs[l][0]), w, h, l, p(T), p(calib), p(curs[l][0]), p(curs[l][1]),
                                           gpad, p(eg), p(jg), p(wpx), 1e-3)
        assert np.array_equal(eg[sel[:n]] != 0, er[:n] != 0), f"icp correspondences level {l}"
        scale = np.abs(er[:n]).max()
        np.testing.assert_allclose(eg[sel[:n]], er[:n], rtol=0, atol=1e-5 * scale)
        for c in range(6):
            col_g = jg[c * gpad:(c + 1) * gpad][sel[:n]]
            col_r = jr[c * npad:c * npad + n]
            np.testing.assert_allclose(col_g, col_r, rtol=0, atol=1e-5 * np.abs(col_r).max(), err_msg=f"J{c} l{l}")


def test_cg_solver_matches_reference():
    rng = np.random.default_rng(0)
    for _ in range(20):
        M = rng.normal(size=(6, 40)).astype(np.float32)
        A = (M @ M.T).astype(np.float32).reshape(-1)
        b = rng.normal(size=6).astype(np.float32)
        xo = np.zeros(6)
        xr = np.zeros(6)
        A64, b64 = A.astype(np.float64), b.astype(np.float64)  # alive across the call
        O.lib().orc_solve_cg(p(A64), p(b64), 1e-8, 6, p(xo))
        R.lib().ref_conjugateGradient(p(A), p(b), p(xr))
        assert np.array_equal(xo, xr)


def test_expm_update_matches_reference_expm():
    rng = np.random.default_rng(1)
    for k in range(50):
        x = (rng.normal(size=6) * np.array([0.05, 0.05, 0.05, 0.03, 0.03, 0.03]) * (0.01 if k % 5 == 0 else 1))
        x = x.astype(np.float32)
        T0 = synth.se3(synth.rodrigues(rng.normal(size=3) * 0.1), rng.normal(size=3) * 50).astype(np.float32)
        To = np.ascontiguousarray(T0).reshape(-1).copy()
        Tr = To.copy()
        x64 = x.astype(np.float64)
        O.lib().orc_expm_update(p(x64), p(To), 1000.0)
        R.lib().ref_expm(p(x), p(Tr), 1000.0)
        # Pade(6) in real vs complex (EXPOKIT) arithmetic: FP64 rounding only
        np.testing.assert_allclose(To, Tr, rtol=0, atol=2e-5 * np.maximum(1, np.abs(Tr)).max())
        assert np.abs(To - Tr).max() <= 4 * np.spacing(np.abs(Tr).max())


def test_canonical_reduction_close_to_reference_order():
    rng = np.random.default_rng(2)
    N = 8192
    J = [rng.normal(size=N).astype(np.float32) for _ in range(6)]
    r = rng.normal(size=N).astype(np.float32)
    A, b = np.zeros(36), np.zeros(6)
    Af, bf = np.zeros(36, np.float32), np.zeros(6, np.float32)
    O.lib().orc_reduce27(O.ptrs(J), p(r), N, p(A), p(b))
    O.lib().orc_reduce27_refordered(O.ptrs(J), p(r), N, p(Af), p(bf))
    Jm = np.stack([j.astype(np.float64) for j in J])
    A_exact = Jm @ Jm.T
    np.testing.assert_allclose(A.reshape(6, 6), A_exact, rtol=1e-5, atol=1e-3)
    np.testing.assert_allclose(Af.reshape(6, 6), A_exact, rtol=1e-5, atol=1e-2)
    np.testing.assert_allclose(b, Jm @ r.astype(np.float64), rtol=1e-5, atol=1e-3)


def test_selection_matches_reference(frame_pair):
    """Pixel selection (A5): the oracle's 256-bin histogram and index list
    equal the reference's extractGradientKernel + seekThreshold256Kernel2 +
    filterIndexKernel4 (filterIndex256.cu:26-46, 110-169), the latter run as
    one block of 512 host threads with its two barriers."""
    fp = frame_pair
    W, H = fp["W"], fp["H"]
    z, xyz_o, xyz_r, lv, vd_o, vd_r = _reference_prep(fp)
    grad = np.ascontiguousarray(vd_o.reshape(-1, 24)[:, 13])
    grad_r = np.zeros(W * H, np.float32)
    R.lib().ref_extractGradient(p(vd_r), W * H, p(grad_r))
    assert np.array_equal(grad.view(np.uint32), grad_r.view(np.uint32))
    hist = np.zeros(256, np.int32)
    O.lib().orc_grad_histogram(p(grad), W * H, 256, p(hist))
    for P in (8192, 4096):
        idx_o = np.zeros(P, np.int32)
        n_o = O.lib().orc_filter_indices(p(grad), W * H, p(hist), 256, P, p(idx_o))
        histf = hist.astype(np.float32)  # cudaHista's float counts
        # the reference's zero-initialised index buffer holds one entry per
        # vertex: the kernel never trims the last of its 512 segments, so it
        # can write past entry P (the tracker then uses the first P)
        idx_r = np.zeros(W * H, np.int32)
        R.lib().ref_filterIndices4(p(grad_r), p(histf), p(idx_r), W * H, P, 256)
        assert np.array_equal(idx_o, idx_r[:P]), P
        # the count the reference writes, P or more (the untrimmed last segment)
        assert n_o >= P
        # the reference's seek wrote the threshold bin and the surplus into hist[0..1]
        thr = int(histf[0])
        assert hist[thr + 1:].sum() <= P < hist[thr:].sum()


def test_rgbd_float4_conversion_matches_reference():
    """Float4 RGBA + normalised depth input (A2): orc_rgbd_float4_to_gray_z
    equals rgbTex2GrayHdrZKernel and rgbdTex2DepthKernel (rgb2gray.cu:64-87)
    reading the frame through a point-sampled texture with the y-flip."""
    W, H = 320, 240
    rng = np.random.default_rng(5)
    rgbd = rng.random((H, W, 4), dtype=np.float32)
    rgbd[..., 3] = rng.random((H, W), dtype=np.float32)
    cal = synth.make_calibration(W, H)
    calib = np.ascontiguousarray(cal.calib, np.float32)
    g_o = np.zeros(W * H, np.float32)
    z_o = np.zeros(W * H, np.float32)
    O.lib().orc_rgbd_float4_to_gray_z(p(rgbd), W, H, p(calib), p(g_o), p(z_o))
    g_r = np.zeros(W * H, np.float32)
    z_r = np.zeros(W * H, np.float32)
    z2_r = np.zeros(W * H, np.float32)
    R.lib().ref_rgbTex2GrayHdrZ(p(rgbd), W, H, p(calib), p(g_r), p(z_r), p(z2_r))
    assert np.array_equal(g_o.view(np.uint32), g_r.view(np.uint32))
    assert np.array_equal(z_o.view(np.uint32), z_r.view(np.uint32))
    assert np.array_equal(z_o.view(np.uint32), z2_r.view(np.uint32))


def _random_poses(n, seed, max_deg, max_mm):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        deg = float(rng.uniform(0.0, max_deg))
        mm = float(rng.uniform(0.0, max_mm))
        out.append(synth.offset_pose(int(rng.integers(1 << 30)), deg, mm).astype(np.float32))
    return out


def test_pose_difference_exceeded_matches_reference():
    """The keyframe trigger (A20): recon_pose_difference_exceeded equals
    PhotoTracker::poseDifferenceExceeded (phototracker.cpp:268-288) compiled
    from the reference, on poses around both thresholds and on identities."""
    import recon_gb300 as rg
    poses = _random_poses(400, 17, 25.0, 250.0) + _random_poses(200, 18, 13.0, 1.0)
    poses += [np.eye(4, dtype=np.float32)]
    eye = np.eye(4, dtype=np.float32)
    eye[:3, 3] = [80.0, 90.0, 30.0]
    poses.append(eye)
    # rotations near 180 degrees take the quaternion's other branches
    for ax in range(3):
        Rm = np.eye(4, dtype=np.float32)
        i, j = [k for k in range(3) if k != ax]
        Rm[i, i] = Rm[j, j] = np.float32(-1.0)
        poses.append(Rm)
    hits = 0
    for T in poses:
        for dist, ang in ((125.0, 12.5), (30.0, 2.0)):
            Tc = np.ascontiguousarray(T.reshape(16))
            a = rg.pose_difference_exceeded(Tc, dist, ang)
            b = bool(R.lib().ref_poseDifferenceExceeded(p(Tc), dist, ang))
            assert a == b, (T, dist, ang)
            hits += a
    assert 0 < hits < 2 * len(poses)


def test_apply_increment_restatement_matches_reference():
    """The Python restatement of applyIncrement used by the GPU test of the
    single tracker's global pose equals the reference's own arithmetic bit for
    bit over a chain of tracked poses."""
    T = np.eye(4, dtype=np.float32)
    G = np.eye(4, dtype=np.float64)
    Tr = np.ascontiguousarray(np.eye(4, dtype=np.float32).reshape(16))
    Gr = np.ascontiguousarray(np.eye(4, dtype=np.float64).reshape(16))
    for Trel in _random_poses(40, 23, 3.0, 40.0):
        T, G = apply_increment_ref_order(T, G, Trel)
        Trel_c = np.ascontiguousarray(Trel.reshape(16))
        R.lib().ref_applyIncrement(p(Tr), p(Gr), p(Trel_c))
        assert np.array_equal(T.reshape(16).view(np.uint32), Tr.view(np.uint32))
        assert np.array_equal(G.reshape(16).view(np.uint64), Gr.view(np.uint64))
