"""The reference-named kernel launchers (include/recon_ref_shim.h) against the oracle.

These entry points keep the reference's names and argument order
(tracker/kernels/cuda_funcs.h:36-111) over its data layouts, so the
reference's PhotoTracker / ShapeTracker call sequences can run on them.  The
test drives them in that order (phototracker.cpp:343-386, 505-511, 646-664;
shapetracker.cpp:357-394) and compares every stage with the oracle bit for bit.
"""
import ctypes

import numpy as np
import pytest

import oracle_lib as O
import recon_gb300 as rg
from scenes import frame_pair

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
vp = ctypes.c_void_p
p = O.ptr


class VBuf(ctypes.Structure):
    _fields_ = [("devPtr", vp), ("indexDevPtr", vp), ("stride", ctypes.c_int32), ("vertexCount", ctypes.c_int32),
                ("elementsCount", ctypes.c_int32)]


class Pyr(ctypes.Structure):
    _fields_ = [("nLayers", ctypes.c_int32), ("width", ctypes.c_int32 * 4), ("height", ctypes.c_int32 * 4),
                ("devPtr", vp * 4)]


def dptr(t):
    return vp(t.data_ptr())


def cuda(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t, dtype=None):
    torch.cuda.synchronize()
    a = t.cpu().numpy()
    return a.view(dtype) if dtype else a


def same(a, b, what):
    a, b = np.ascontiguousarray(a), np.ascontiguousarray(b)
    assert a.shape == b.shape, what
    va = a.view(np.uint32) if a.dtype == np.float32 else a
    vb = b.view(np.uint32) if b.dtype == np.float32 else b
    assert np.array_equal(va, vb), f"{what}: {np.count_nonzero(va != vb)} differ"


@pytest.fixture(scope="module")
def L():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return rg.lib()


def status(L):
    L.recon_last_status.restype = ctypes.c_int
    return L.recon_last_status()


@pytest.mark.parametrize("W,H,levels", [(320, 240, 3), (640, 480, 4)])
def test_photometric_call_sequence(L, W, H, levels):
    pr = frame_pair(W, H, levels, seed=91, distortion=(levels == 4))
    calib = cuda(pr.cal.calib)
    n = W * H
    P = 8192
    # gray pyramids (downSample2Pyramid) for reference and current
    g_ref = [cuda((pr.g0.astype(np.float32) / np.float32(255.0)).reshape(-1))]
    g_cur = [cuda((pr.g1.astype(np.float32) / np.float32(255.0)).reshape(-1))]
    for l in range(1, levels):
        g_ref.append(torch.zeros((W >> l) * (H >> l), device="cuda"))
        g_cur.append(torch.zeros((W >> l) * (H >> l), device="cuda"))
    pyr_ref, pyr_cur = Pyr(), Pyr()
    for pyr, imgs in ((pyr_ref, g_ref), (pyr_cur, g_cur)):
        pyr.nLayers = levels
        for l in range(levels):
            pyr.width[l], pyr.height[l] = W >> l, H >> l
            pyr.devPtr[l] = imgs[l].data_ptr()
        L.downSample2Pyramid(ctypes.byref(pyr), None)
        assert status(L) == 0
    orc = O.OracleTracker(O.make_config(W, H, levels, mode=O.PHOTOMETRIC), pr.cal.calib)
    orc.set_reference(pr.g0, pr.d0)
    orc.set_current(pr.g1, pr.d1)
    for l in range(levels):
        nl = (W >> l) * (H >> l)
        same(host(g_ref[l]), orc.get("ref_gray", l, nl, np.float32), f"ref pyramid {l}")
        same(host(g_cur[l]), orc.get("cur_gray", l, nl, np.float32), f"cur pyramid {l}")
    zref = cuda(np.where(pr.d0 > 0, -pr.d0.astype(np.float32), 0).astype(np.float32).reshape(-1))
    zcur = cuda(np.where(pr.d1 > 0, -pr.d1.astype(np.float32), 0).astype(np.float32).reshape(-1))
    xyz = torch.zeros(4 * n, device="cuda")
    L.convertZmapToXYZCuda(dptr(zref), dptr(xyz), dptr(calib), W, H, None)
    vdata = torch.zeros(24 * n, device="cuda")
    idx = torch.zeros(n, dtype=torch.int32, device="cuda")
    vb = VBuf(vdata.data_ptr(), idx.data_ptr(), 24, 0, 0)
    L.xyz2CloudCuda(dptr(xyz), dptr(calib), ctypes.byref(vb), ctypes.byref(pyr_ref), None)
    grad = torch.zeros(n, device="cuda")
    L.extractGradientMagnitudes(ctypes.byref(vb), dptr(grad), None)
    hist = torch.zeros(256, device="cuda")
    L.cudaHista.restype = ctypes.c_double
    L.cudaHista(dptr(grad), dptr(hist), n, 256, None, None)
    L.filterIndices4(ctypes.byref(vb), dptr(grad), dptr(hist), P, 256, None)
    assert vb.elementsCount == P and status(L) == 0
    L.addVertexAttributesWithoutNormalsCuda(dptr(calib), ctypes.byref(vb), ctypes.byref(pyr_ref), None)
    J = [torch.zeros(6 * P, device="cuda") for _ in range(4)]
    L.precomputeJacobian4Cuda(ctypes.byref(vb), dptr(calib), *[dptr(j) for j in J], ctypes.c_float(1e-3), None)
    assert status(L) == 0
    same(host(idx)[:P], orc.get("sel_idx", 0, P, np.int32), "selected indices")
    rec = host(vdata).reshape(n, 24)[host(idx)[:P]]
    same(np.ascontiguousarray(rec[:, :3].T).reshape(-1), orc.get("sel_xyz", 0, 3 * P, np.float32), "xyz")
    for l in range(levels):
        same(rec[:, [14, 17, 20, 23][l]], orc.get("sel_I", l, P, np.float32), f"intensity {l}")
        same(host(J[l]), orc.get("sel_J", l, 6 * P, np.float32), f"jacobian {l}")
    # one photometric iteration at every level (updateLinearSystem + estimateIncrement)
    T = cuda(np.eye(4, dtype=np.float32).reshape(-1))
    res, zw, w, wr = (torch.zeros(P, device="cuda") for _ in range(4))
    Jw = torch.zeros(6 * P, device="cuda")
    JtJ, b6 = torch.zeros(36, device="cuda"), torch.zeros(6, device="cuda")
    pyr_cur_full = pyr_cur
    for l in range(levels - 1, -1, -1):
        L.interpolateResidual2(ctypes.byref(vb), dptr(T), dptr(calib), ctypes.byref(pyr_cur_full), l, dptr(zcur),
                               dptr(zw), dptr(res), None)
        L.generateWeights64(dptr(res), P, dptr(w), dptr(zw), dptr(wr), None)
        L.weightJacobian(dptr(J[l]), dptr(w), P, dptr(Jw), None)
        L.JTJCuda(dptr(Jw), P, dptr(JtJ), None)
        L.JTresidualCuda(dptr(Jw), dptr(wr), P, dptr(b6), None)
        # the oracle's same iteration
        To = host(T).copy()
        sel_xyz = orc.get("sel_xyz", 0, 3 * P, np.float32)
        I = orc.get("sel_I", l, P, np.float32)
        ro, zo = np.zeros(P, np.float32), np.zeros(P, np.float32)
        cur = orc.get("cur_gray", l, (W >> l) * (H >> l), np.float32)
        zc = orc.get("cur_z", 0, n, np.float32)
        O.lib().orc_interpolate_residual(P, p(sel_xyz), p(I), p(To), p(pr.cal.calib), l, p(cur), W >> l, H >> l,
                                         p(zc), W, H, p(ro), p(zo))
        same(host(res), ro, f"residual {l}")
        same(host(zw), zo, f"zweight {l}")
        ho, wo, rwo = np.zeros(64, np.int32), np.zeros(P, np.float32), np.zeros(P, np.float32)
        O.lib().orc_generate_weights(p(ro), p(zo), P, 64, p(ho), p(wo), p(rwo))
        same(host(w), wo, f"weights {l}")
        same(host(wr), rwo, f"weighted residual {l}")
        Jo = orc.get("sel_J", l, 6 * P, np.float32).reshape(6, P) * wo[None, :]
        Ao, bo = np.zeros(36), np.zeros(6)
        Jcols = [np.ascontiguousarray(Jo[c]) for c in range(6)]  # kept alive across the call
        O.lib().orc_reduce27(O.ptrs(Jcols), p(rwo), P, p(Ao), p(bo))
        same(host(JtJ), Ao.astype(np.float32), f"JtJ {l}")
        same(host(b6), bo.astype(np.float32), f"Jtr {l}")
        L.solveMotionCuda(dptr(JtJ), dptr(b6), dptr(T), ctypes.c_float(1000.0), None)
        xo = np.zeros(6)
        Af = Ao.astype(np.float32).astype(np.float64)  # the float system solveMotionCuda receives
        bf = bo.astype(np.float32).astype(np.float64)
        O.lib().orc_solve_cg(p(Af), p(bf), 1e-8, 6, p(xo))
        O.lib().orc_expm_update(p(xo), p(To), 1000.0)
        same(host(T), To, f"pose after level {l}")


def test_icp_call_sequence(L):
    W, H, levels = 320, 240, 3
    pr = frame_pair(W, H, levels, seed=92)
    calib = cuda(pr.cal.calib)
    orc = O.OracleTracker(O.make_config(W, H, levels, mode=O.GEOMETRIC), pr.cal.calib)
    orc.set_reference(pr.g0, pr.d0)
    orc.set_current(pr.g1, pr.d1)
    n = W * H
    zref = cuda(np.where(pr.d0 > 0, -pr.d0.astype(np.float32), 0).astype(np.float32).reshape(-1))
    zcur = cuda(np.where(pr.d1 > 0, -pr.d1.astype(np.float32), 0).astype(np.float32).reshape(-1))
    ref = [torch.zeros(6 * (n >> (2 * l)), device="cuda") for l in range(levels)]
    cur = [torch.zeros(6 * (n >> (2 * l)), device="cuda") for l in range(levels)]
    rm = [torch.zeros(n >> (2 * l), dtype=torch.int32, device="cuda") for l in range(levels)]
    cm = [torch.zeros(n >> (2 * l), dtype=torch.int32, device="cuda") for l in range(levels)]
    L.convertZmapToXYZ6Cuda(dptr(zref), dptr(ref[0]), dptr(rm[0]), dptr(calib), W, H, None)
    L.computeNormals6Cuda(dptr(ref[0]), dptr(rm[0]), W, H, None)
    L.genPointCloud6Cuda(dptr(zcur), W, H, dptr(cur[0]), dptr(cm[0]), dptr(calib), None)
    for l in range(1, levels):
        L.downSampleCloud6Cuda(dptr(ref[l - 1]), dptr(rm[l - 1]), dptr(ref[l]), dptr(rm[l]), W >> l, H >> l, None)
        L.downSampleCloud6Cuda(dptr(cur[l - 1]), dptr(cm[l - 1]), dptr(cur[l]), dptr(cm[l]), W >> l, H >> l, None)
    for l in range(levels):
        nl = n >> (2 * l)
        same(host(rm[l]), orc.get("refmask", l, nl, np.int32), f"ref mask {l}")
        same(host(ref[l]), orc.get("ref6", l, 6 * nl, np.float32), f"ref cloud {l}")
        same(host(cm[l]), orc.get("curmask", l, nl, np.int32), f"cur mask {l}")
        same(host(cur[l]), orc.get("cur6", l, 6 * nl, np.float32), f"cur cloud {l}")
    T = np.ascontiguousarray((0.5 * (np.eye(4) + pr.T_gt)).astype(np.float32)).reshape(-1)
    Td = cuda(T)
    for l in range(levels):
        w, h = W >> l, H >> l
        nl = w * h
        full, rmask = torch.zeros(nl, device="cuda"), torch.zeros(nl, dtype=torch.int32, device="cuda")
        L.icpResidualMaskCuda2(dptr(ref[l]), dptr(rm[l]), w, h, dptr(Td), dptr(calib), dptr(cur[l]), dptr(cm[l]), l,
                               dptr(full), dptr(rmask), None)
        part = torch.zeros(1024, dtype=torch.int32, device="cuda")
        sel = torch.zeros(nl, dtype=torch.int32, device="cuda")
        L.selectValidIndex(dptr(rmask), nl, dptr(part), 1024, dptr(sel), None)
        nsel = int(host(part)[0])
        r, r2, wts = (torch.zeros(max(nsel, 1), device="cuda") for _ in range(3))
        L.packIndex(dptr(sel), nsel, dptr(full), dptr(r), dptr(r2), None)
        psum = torch.zeros(1024, device="cuda")
        L.generateStudentTWeights(dptr(r2), nsel, dptr(psum), 1024, dptr(wts), None)
        npad = ((nsel + 1023) // 1024) * 1024
        res, J = torch.zeros(npad, device="cuda"), torch.zeros(6 * npad, device="cuda")
        L.icpResidualCuda2(dptr(ref[l]), dptr(sel), nsel, w, h, l, dptr(Td), dptr(calib), dptr(cur[l]), dptr(cm[l]),
                           npad, dptr(res), dptr(J), dptr(wts), ctypes.c_float(1e-3), None)
        assert status(L) == 0
        # oracle (arrays bound to names so that they outlive the calls)
        o_ref6, o_rm = orc.get("ref6", l, 6 * nl, np.float32), orc.get("refmask", l, nl, np.int32)
        o_cur6, o_cm = orc.get("cur6", l, 6 * nl, np.float32), orc.get("curmask", l, nl, np.int32)
        ofull, omask = np.zeros(nl, np.float32), np.zeros(nl, np.int32)
        O.lib().orc_icp_residual_mask(p(o_ref6), p(o_rm), w, h, p(T), p(pr.cal.calib), p(o_cur6), p(o_cm), l,
                                      p(ofull), p(omask))
        same(host(rmask), omask, f"icp mask {l}")
        osel = np.zeros(nl, np.int32)
        on = O.lib().orc_compact(p(omask), nl, p(osel))
        assert nsel == on
        same(host(sel)[:nsel], osel[:on], f"compaction {l}")
        orv = ofull[osel[:on]]
        or2 = (orv * orv).astype(np.float32)
        ow = np.zeros(on, np.float32)
        O.lib().orc_student_t(p(or2), on, p(ow))
        same(host(wts)[:nsel], ow, f"student-t {l}")
        ores, oJ = np.zeros(npad, np.float32), np.zeros(6 * npad, np.float32)
        O.lib().orc_icp_residual_jacobian(p(o_ref6), p(osel), on, w, h, l, p(T), p(pr.cal.calib), p(o_cur6),
                                          p(o_cm), npad, p(ores), p(oJ), p(ow), 1e-3)
        same(host(res), ores, f"icp residual {l}")
        same(host(J), oJ, f"icp jacobian {l}")


def test_linear_fuse(L):
    rng = np.random.default_rng(3)
    A1, A2 = rng.normal(size=36).astype(np.float32), rng.normal(size=36).astype(np.float32)
    b1, b2 = rng.normal(size=6).astype(np.float32), rng.normal(size=6).astype(np.float32)
    dA1, db1, dA2, db2 = cuda(A1), cuda(b1), cuda(A2), cuda(b2)  # all alive during the launch
    L.linearFuseCuda(dptr(dA1), dptr(db1), ctypes.c_float(0.5), 8192, dptr(dA2), dptr(db2),
                     ctypes.c_float(0.5), 5000, None)
    i1, i2 = np.float32(1.0 / 8192.0), np.float32(1.0 / 5000.0)
    w = np.float32(0.5)
    same(host(dA1), (i1 * w * A1 + i2 * w * A2).astype(np.float32), "fused A")
    same(host(db1), (i1 * w * b1 + i2 * w * b2).astype(np.float32), "fused b")
