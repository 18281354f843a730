"""End-to-end gap between this tracker and the reference's own pipeline (CPU).

RefTracker chains the reference's own code, compiled from its sources into
oracle/_ref, in the order PhotoTracker / ShapeTracker call it
(phototracker.cpp:338-386, 505-511, 646-689; shapetracker.cpp:205-288,
357-394): xyz2CloudKernel, extractGradientKernel, filterIndexKernel4,
addVertexAttributesWithoutNormalsKernel3/4, precomputeJacobian4Kernel,
interpolateResidualKernel2, the 64-bin weights, weightJacobianKernel, the
ICP cloud and normal kernels, icpResidualKernel2, packIndexKernel, the
Student-t passes, icpResidualIndexKernel2, linearFuseKernel,
conjugateGradientKernel and expm.  Three steps are not the reference's
compiled code: the 256-bin gradient histogram (its bin formula, gpu_hist.cu:136,
counted exactly), the stable compaction of the ICP mask (selectValidIndex,
rgb2gray.cu:393-460: the set bits in index order) and the FP32 normal
equations, summed in the reference's order (JTJCuda / JTresidualCuda,
warp.cu:1430-1487; reduction_kernel.cu:262-340) by orc_reduce27_refordered.
The SE(3) update is the reference's CPU expm.c (expm(x, T)), which takes the
increment as float where expmKernel takes it as double.

The tracker here (GPU, bit-identical to the FP32 oracle) departs from that
pipeline on purpose in the normal equations (exact fixed-point sums kept in
FP64), the solve (FP64 LDL^T by default; the reference's CG on request), the
exponential (real Pade in FP64) and the fused multiply-adds of the ICP
Jacobian; the per-pixel values match the reference (tests/test_oracle_pin.py).
This test runs both on the same frames and fixed schedules and bounds the
final pose gap; the measured gaps are stated in the design notes.
"""
import ctypes

import numpy as np
import pytest

import oracle_lib as O
import ref_lib as R
from recon_gb300 import synth
from scenes import frame_pair

pytestmark = pytest.mark.skipif(not R.available(), reason="reference tree not built into oracle/_ref")

p = O.ptr


def _pad1024(n):
    return ((n + 1023) // 1024) * 1024


class RefTracker:
    """The reference's pipeline from its own kernels (see the module docstring)."""

    def __init__(self, W, H, L, calib, mode, iters, P=8192, lam=0.5, hist_bins=64):
        assert hist_bins == 64  # generateWeights64: the reference's MAD histogram
        self.W, self.H, self.L, self.P, self.mode, self.iters, self.lam = W, H, L, P, mode, iters, lam
        self.calib = np.ascontiguousarray(calib, np.float32)
        self.o, self.r = O.lib(), R.lib()

    def _gray_pyramid(self, g8):
        lv = [np.ascontiguousarray(g8.reshape(-1).astype(np.float32) / np.float32(255.0))]
        for l in range(1, self.L):
            lo = np.zeros((self.W >> l) * (self.H >> l), np.float32)
            self.r.ref_fastDownSampleHdr(p(lv[-1]), self.W >> l, self.H >> l, p(lo))
            lv.append(lo)
        return lv

    def _z(self, d16):
        z = np.zeros(self.W * self.H, np.float32)
        d = np.ascontiguousarray(d16.reshape(-1), np.uint16)
        self.o.orc_convert_depth(p(d), self.W * self.H, p(z))
        return z

    def _cloud_pyramid(self, top, mask):
        out = [(top, mask)]
        for l in range(1, self.L):
            w, h = self.W >> l, self.H >> l
            d, m = np.zeros(6 * w * h, np.float32), np.zeros(w * h, np.int32)
            self.r.ref_downSampleCloud6(p(out[-1][0]), p(out[-1][1]), p(d), p(m), w, h)
            out.append((d, m))
        return out

    def set_reference(self, g8, d16):
        W, H, L, P, r = self.W, self.H, self.L, self.P, self.r
        lv = self._gray_pyramid(g8)
        z = self._z(d16)
        xyz = np.zeros(4 * W * H, np.float32)
        r.ref_convertZMapToXYZ(p(z), p(xyz), p(self.calib), W, H)
        self.vd = np.zeros(24 * W * H, np.float32)
        r.ref_xyz2Cloud(p(xyz), W, H, p(self.calib), p(self.vd), p(lv[0]))
        grad = np.zeros(W * H, np.float32)
        r.ref_extractGradient(p(self.vd), W * H, p(grad))
        hist = np.zeros(256, np.int32)
        self.o.orc_grad_histogram(p(grad), W * H, 256, p(hist))
        histf = hist.astype(np.float32)
        idx = np.zeros(W * H, np.int32)
        r.ref_filterIndices4(p(grad), p(histf), p(idx), W * H, P, 256)
        self.idx = np.ascontiguousarray(idx[:P])
        # padded gray copies: the 4-level attribute kernel reads up to one
        # row/column outside the coarsest image
        pad = 4 * (W >> 1)
        self._pads = []
        for l in range(L):
            buf = np.zeros(lv[l].size + 2 * pad, np.float32)
            buf[pad:pad + lv[l].size] = lv[l]
            self._pads.append(buf)
        gp = [ctypes.c_void_p(b.ctypes.data + 4 * pad) for b in self._pads] + [ctypes.c_void_p(0)] * (4 - L)
        r.ref_addVertexAttributes(p(self.idx), P, p(self.vd), W, H, p(self.calib), *gp, L)
        self.J = [np.zeros(6 * P, np.float32) for _ in range(4)]
        r.ref_precomputeJacobian4(p(self.idx), P, p(self.vd), p(self.calib), *[p(j) for j in self.J], 1e-3)
        pts, m = np.zeros(6 * W * H, np.float32), np.zeros(W * H, np.int32)
        r.ref_convertZMapToXYZ6(p(z), p(pts), p(m), p(self.calib), W, H)
        r.ref_computeNormals(p(pts), p(m), W, H)
        self.ref6 = self._cloud_pyramid(pts, m)
        self.T = np.eye(4, dtype=np.float32).reshape(16).copy()

    def set_current(self, g8, d16):
        self.cur = self._gray_pyramid(g8)
        self.zc = self._z(d16)
        pts, m = np.zeros(6 * self.W * self.H, np.float32), np.zeros(self.W * self.H, np.int32)
        self.r.ref_genPointsCloud6(p(self.zc), self.W, self.H, p(self.calib), p(pts), p(m))
        self.cur6 = self._cloud_pyramid(pts, m)

    def _photometric(self, layer):
        P, r = self.P, self.r
        w, h = self.W >> layer, self.H >> layer
        res, zw = np.zeros(P, np.float32), np.zeros(P, np.float32)
        r.ref_interpolateResidual2(p(self.idx), P, p(self.vd), p(self.T), p(self.calib), layer, p(self.cur[layer]),
                                   w, h, p(self.zc), self.W, self.H, p(res), p(zw))
        wt, wres, hist = np.zeros(P, np.float32), np.zeros(P, np.float32), np.zeros(64, np.int32)
        r.ref_generateWeights64(p(res), P, p(wt), p(zw), p(wres), p(hist))
        Jw = np.zeros(6 * P, np.float32)
        r.ref_weightJacobian(p(self.J[layer]), p(wt), P, p(Jw))
        cols = [np.ascontiguousarray(Jw[c * P:(c + 1) * P]) for c in range(6)]
        A, b = np.zeros(36, np.float32), np.zeros(6, np.float32)
        self.o.orc_reduce27_refordered(O.ptrs(cols), p(wres), P, p(A), p(b))
        return A, b

    def _icp(self, layer, j):
        r = self.r
        w, h = self.W >> layer, self.H >> layer
        (ref6, rmask), (cur6, cmask) = self.ref6[layer], self.cur6[layer]
        if j == 0:
            full, msk = np.zeros(w * h, np.float32), np.zeros(w * h, np.int32)
            r.ref_icpResidualMask2(p(ref6), p(rmask), w, h, p(self.T), p(self.calib), p(cur6), p(cmask), layer,
                                   p(full), p(msk))
            self.sel = np.ascontiguousarray(np.flatnonzero(msk > 0).astype(np.int32))
            self.nsel = int(self.sel.size)
            if self.nsel <= 0:
                return None
            rr, r2 = np.zeros(self.nsel, np.float32), np.zeros(self.nsel, np.float32)
            r.ref_packIndex(p(self.sel), self.nsel, p(full), p(rr), p(r2))
            self.wicp = np.zeros(self.nsel, np.float32)
            r.ref_studentT(p(r2), self.nsel, p(self.wicp))
        if self.nsel <= 0:
            return None
        npad = _pad1024(self.nsel)
        res, J = np.zeros(npad, np.float32), np.zeros(6 * npad, np.float32)
        r.ref_icpResidual2(p(ref6), p(self.sel), self.nsel, w, h, layer, p(self.T), p(self.calib), p(cur6), p(cmask),
                           npad, p(res), p(J), p(self.wicp), 1e-3)
        cols = [np.ascontiguousarray(J[c * npad:(c + 1) * npad]) for c in range(6)]
        A, b = np.zeros(36, np.float32), np.zeros(6, np.float32)
        self.o.orc_reduce27_refordered(O.ptrs(cols), p(res), npad, p(A), p(b))
        return A, b

    def track(self, T0=None):
        if T0 is not None:
            self.T = np.array(T0, np.float32).reshape(16).copy()
        L = self.L
        for layer in range(L - 1, -1, -1):
            for j in range(self.iters[L - 1 - layer]):
                ph = self._photometric(layer) if self.mode != O.GEOMETRIC else None
                icp = self._icp(layer, j) if self.mode != O.PHOTOMETRIC else None
                if self.mode != O.PHOTOMETRIC and icp is None:
                    continue  # "not enough points": no solve
                if self.mode == O.PHOTOMETRIC:
                    A, b = ph
                elif self.mode == O.GEOMETRIC:
                    A, b = icp
                else:
                    A, b = ph
                    iN1 = np.float32(1.0 / float(self.P))
                    iN2 = np.float32(1.0 / float(self.nsel))
                    self.r.ref_linearFuse(p(A), p(b), 1.0 - self.lam, iN1, p(icp[0]), p(icp[1]), self.lam, iN2)
                x = np.zeros(6, np.float64)
                self.r.ref_conjugateGradient(p(A), p(b), p(x))
                xf = x.astype(np.float32)
                self.r.ref_expm(p(xf), p(self.T), 1000.0)
        return self.T.reshape(4, 4).copy()


CASES = [
    # config 1: one 320x240 pair, photometric, 10 GN iterations per level (64-bin MAD)
    dict(W=320, H=240, L=3, mode=O.PHOTOMETRIC, iters=(10, 10, 10), seed=2024, distortion=False),
    # a 640x480 bi-objective pair with lens distortion on the reference schedule
    dict(W=640, H=480, L=4, mode=O.BIOBJECTIVE, iters=(1, 3, 10, 5), seed=31, distortion=True),
]


def _run(case, solver):
    pr = frame_pair(case["W"], case["H"], case["L"], seed=case["seed"], distortion=case["distortion"])
    ref = RefTracker(case["W"], case["H"], case["L"], pr.cal.calib, case["mode"], case["iters"])
    ref.set_reference(pr.g0, pr.d0)
    ref.set_current(pr.g1, pr.d1)
    Tr = ref.track()
    cfg = O.make_config(case["W"], case["H"], case["L"], mode=case["mode"], iters=case["iters"], solver=solver)
    orc = O.OracleTracker(cfg, pr.cal.calib)
    orc.set_reference(pr.g0, pr.d0)
    orc.set_current(pr.g1, pr.d1)
    To, _ = orc.track()
    o64 = O.Oracle64Tracker(cfg, pr.cal.calib)
    o64.set_reference(pr.g0, pr.d0)
    o64.set_current(pr.g1, pr.d1)
    T64 = o64.track()
    return pr, Tr.astype(np.float64), To.astype(np.float64), T64


@pytest.mark.parametrize("case", CASES, ids=["config1_320x240_photometric", "640x480_biobjective"])
def test_tracker_pose_close_to_reference_pipeline(case):
    """The tracker's final pose (the oracle's, which the GPU reproduces bit for
    bit) against the reference-ordered pipeline on the same inputs, with the
    reference's CG solver and with the default FP64 LDL^T: within the
    tracking contract of 1e-6 m and 1e-6 rad over the fixed schedule
    (measured: 3.7e-4 mm / 1.8e-6 deg for config 1, 5.1e-4 mm / 3.9e-6 deg
    (CG) and 5.7e-4 mm / 1.8e-5 deg (LDL^T) for the 640x480 pair).  The
    reference pipeline itself is within 0.01 mm / 0.0005 deg of the FP64
    oracle."""
    tol_mm, tol_deg = 1e-6 * 1e3, float(np.degrees(1e-6))
    for solver in (O.CG, O.CHOLESKY):
        pr, Tr, To, T64 = _run(case, solver)
        mm, deg = synth.pose_error(To, Tr)
        print(f"{case['W']}x{case['H']} solver {solver}: tracker vs reference pipeline {mm:.3e} mm {deg:.3e} deg")
        assert mm < tol_mm and deg < tol_deg, (solver, mm, deg)
    mm, deg = synth.pose_error(Tr, T64)
    print(f"reference pipeline vs FP64 oracle {mm:.3e} mm {deg:.3e} deg")
    assert mm < 1e-2 and deg < 5e-4, (mm, deg)
