"""C-ABI checks that need no GPU: the library loads, exports every function that
the headers under include/ declare, and its host-only entry points behave."""
import ctypes
import os
import re

import numpy as np
import pytest

import oracle_lib as O
import recon_gb300 as rg
from recon_gb300 import build, synth

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def L():
    build.build()
    return rg.lib()


def declared_functions(header=None):
    names = set()
    inc = os.path.join(ROOT, "include")
    for h in sorted(os.listdir(inc)) if header is None else [header]:
        if not h.endswith(".h"):
            continue
        src = open(os.path.join(inc, h)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names |= set(re.findall(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\**\s*(recon_[a-z0-9_]+)\s*\(", src,
                                flags=re.M))
    return sorted(names)


def test_header_declares_the_operator_api():
    names = declared_functions("recon_track.h")
    for required in ["recon_tracker_create", "recon_set_reference", "recon_set_current", "recon_track",
                     "recon_set_iterations", "recon_set_mode", "recon_reset", "recon_get_global_pose",
                     "recon_batch_create", "recon_batch_track", "recon_calib_setup"]:
        assert required in names
    tsdf = declared_functions("recon_tsdf.h")
    for required in ["recon_tsdf_create", "recon_tsdf_reset", "recon_tsdf_update", "recon_tsdf_raycast",
                     "recon_tsdf_resample", "recon_tsdf_set_dist_rgbd_float4", "recon_tsdf_device_array"]:
        assert required in tsdf


def test_library_exports_every_declared_symbol(L):
    out = os.popen(f"nm -D --defined-only {rg.LIB_PATH}").read()
    exported = set(re.findall(r" T (\w+)", out))
    missing = [n for n in declared_functions() if n not in exported]
    assert not missing, missing
    for n in declared_functions():
        assert hasattr(L, n)


def test_calib_setup_matches_oracle_and_python(L):
    for W, dist in [(320, False), (640, True), (80, False)]:
        cal = synth.make_calibration(W, W * 3 // 4, distortion=dist)
        KL = np.ascontiguousarray(cal.KL, np.float64)
        KR = np.ascontiguousarray(cal.KR, np.float64)
        TLR = np.ascontiguousarray(cal.TLR.reshape(-1), np.float64)
        kc = np.ascontiguousarray(cal.kcR, np.float64)
        out = np.zeros(96, np.float32)
        c1, c0 = float(cal.calib[42]), float(cal.calib[61])
        rg.check(L.recon_calib_setup(O.ptr(KL), O.ptr(KR), O.ptr(TLR), O.ptr(kc), cal.min_dist, cal.max_dist,
                                     c0, c1, W, O.ptr(out)))
        orc = np.zeros(96, np.float32)
        O.lib().orc_calib_setup.argtypes = [ctypes.c_void_p] * 4 + [ctypes.c_double] * 4 + [ctypes.c_int,
                                                                                             ctypes.c_void_p]
        O.lib().orc_calib_setup(O.ptr(KL), O.ptr(KR), O.ptr(TLR), O.ptr(kc), cal.min_dist, cal.max_dist, c0, c1,
                                W, O.ptr(orc))
        on_path = np.r_[0:9, 18:43, 43:52, 62:80]
        assert np.array_equal(out[on_path].view(np.uint32), orc[on_path].view(np.uint32))
        assert np.array_equal(out[on_path].view(np.uint32), cal.calib[on_path].view(np.uint32))


def test_invalid_arguments_are_rejected(L):
    cfg = rg.make_config(320, 240)
    h = ctypes.c_void_p()
    cal = np.zeros(96, np.float32)
    assert L.recon_batch_create(0, ctypes.byref(cfg), O.ptr(cal), None, ctypes.byref(h)) == -1
    assert L.recon_batch_create(1, None, O.ptr(cal), None, ctypes.byref(h)) == -1
    assert L.recon_batch_destroy(None) == 0
    assert L.recon_track(None, None, None) == -1
    assert L.recon_calib_setup(None, None, None, None, 0.0, 0.0, 0.0, 0.0, 0, None) == -1


def test_no_device_is_reported_not_faked(L):
    if L.recon_device_count() > 0:
        pytest.skip("a GPU is present")
    cfg = rg.make_config(320, 240)
    h = ctypes.c_void_p()
    cal = synth.make_calibration(320, 240).calib
    rc = L.recon_batch_create(1, ctypes.byref(cfg), O.ptr(cal), None, ctypes.byref(h))
    assert rc == -7
    with pytest.raises(rg.ReconError):
        rg.Tracker(cfg, cal)
