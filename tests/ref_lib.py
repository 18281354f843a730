"""ctypes binding of oracle/_ref/libreconref.so (the reference's own kernels built for the host).

Test infrastructure.  The library exists only where the reference tree was
available at build time (oracle/build_ref.py); tests that need it skip otherwise.
"""
from __future__ import annotations

import ctypes
import os

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_LIB = os.path.join(ROOT, "oracle", "_ref", "libreconref.so")

_lib = None


def available() -> bool:
    return os.path.exists(REF_LIB)


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        L = ctypes.CDLL(REF_LIB)
        vp, i32, f32 = ctypes.c_void_p, ctypes.c_int, ctypes.c_float
        L.ref_convertZMapToXYZ.argtypes = [vp, vp, vp, i32, i32]
        L.ref_convertZMapToXYZ6.argtypes = [vp, vp, vp, vp, i32, i32]
        L.ref_xyz2Cloud.argtypes = [vp, i32, i32, vp, vp, vp]
        L.ref_extractGradient.argtypes = [vp, i32, vp]
        L.ref_addVertexAttributes.argtypes = [vp, i32, vp, i32, i32, vp, vp, vp, vp, vp, i32]
        L.ref_precomputeJacobian4.argtypes = [vp, i32, vp, vp, vp, vp, vp, vp, f32]
        L.ref_interpolateResidual2.argtypes = [vp, i32, vp, vp, vp, i32, vp, i32, i32, vp, i32, i32, vp, vp]
        L.ref_generateWeights64.argtypes = [vp, i32, vp, vp, vp, vp]
        L.ref_generateWeights64.restype = i32
        L.ref_weightJacobian.argtypes = [vp, vp, i32, vp]
        L.ref_fastDownSampleHdr.argtypes = [vp, i32, i32, vp]
        L.ref_genPointsCloud6.argtypes = [vp, i32, i32, vp, vp, vp]
        L.ref_computeNormals.argtypes = [vp, vp, i32, i32]
        L.ref_downSampleCloud6.argtypes = [vp, vp, vp, vp, i32, i32]
        L.ref_icpResidualMask2.argtypes = [vp, vp, i32, i32, vp, vp, vp, vp, i32, vp, vp]
        L.ref_icpResidual2.argtypes = [vp, vp, i32, i32, i32, i32, vp, vp, vp, vp, i32, vp, vp, vp, f32]
        L.ref_packIndex.argtypes = [vp, i32, vp, vp, vp]
        L.ref_studentT.argtypes = [vp, i32, vp]
        L.ref_conjugateGradient.argtypes = [vp, vp, vp]
        L.ref_linearFuse.argtypes = [vp, vp, f32, f32, vp, vp, f32, f32]
        L.ref_expm.argtypes = [vp, vp, f32]
        L.ref_filterIndices4.argtypes = [vp, vp, vp, i32, i32, i32]
        L.ref_rgbTex2GrayHdrZ.argtypes = [vp, i32, i32, vp, vp, vp, vp]
        L.ref_poseDifferenceExceeded.argtypes = [vp, f32, f32]
        L.ref_poseDifferenceExceeded.restype = i32
        L.ref_applyIncrement.argtypes = [vp, vp, vp]
        L.ref_genOrientedPoints6.argtypes = [vp, vp, i32, i32, vp, vp, vp]
        L.ref_d2Z.argtypes = [vp, i32, i32, f32, f32, f32, f32, f32, f32, vp]
        L.ref_d2ZLow.argtypes = [vp, i32, i32, f32, f32, f32, f32, f32, f32, vp]
        L.ref_convert2Gray.argtypes = [vp, i32, i32, vp]
        L.ref_undistort.argtypes = [vp, i32, i32, vp, vp, vp, i32, vp]
        L.ref_undistortDisparity.argtypes = [vp, vp, i32, i32, vp]
        L.ref_d2ZLowGpu.argtypes = [vp, vp, i32, i32, vp, f32, f32]
        L.ref_d2ZLowHdrGpu.argtypes = [vp, vp, i32, i32, vp, f32, f32]
        L.ref_convertHdrRGB.argtypes = [vp, vp, i32, i32]
        L.ref_rgb2GrayHdr.argtypes = [vp, vp, i32, i32]
        L.ref_rgbF2GrayHdr.argtypes = [vp, vp, i32, i32]
        L.ref_undistortHdrRGB.argtypes = [vp, vp, i32, i32, vp]
        L.ref_result_save.argtypes = [ctypes.c_char_p, vp, i32, i32, i32, i32]
        L.ref_track_params_get.argtypes = [ctypes.c_char_p, i32, vp, vp, vp]
        L.ref_tsdf_reset.argtypes = [vp, i32]
        L.ref_tsdf_reconstruction.argtypes = [vp, i32, i32, f32, f32, vp]
        L.ref_tsdf_update.argtypes = [vp, i32, vp, vp, i32, i32, f32, f32, vp, vp, vp]
        L.ref_tsdf_raycast.argtypes = [vp, i32, vp, vp, i32, i32, f32, f32, vp, vp, i32, vp]
        L.ref_tsdf_shade.argtypes = [vp, i32, i32, vp, vp]
        L.ref_tsdf_resample.argtypes = [vp, vp, i32, vp, vp, vp]
        _lib = L
    return _lib
