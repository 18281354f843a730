"""The reference's result files (CPU): the trajectory file of ResultTxt and the
per-segment mode list of TrackingParams, written and read by the library and
compared byte for byte / entry for entry with the reference's own classes
(tracker/calib/ResultTxt.cpp, TrackingParams.cpp, built by oracle/build_ref.py)."""
import os

import numpy as np
import pytest

import oracle_lib as O
import recon_gb300 as rg
import ref_lib as RL
from recon_gb300 import synth

needs_ref = pytest.mark.skipif(not RL.available(), reason="oracle/_ref not built (reference tree absent)")
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def trajectory(n=40, seed=3):
    poses = synth.smooth_trajectory(n, seed, max_step_mm=30.0, max_step_deg=2.0)
    # an arbitrary first pose, as a global pose seldom starts at the identity
    T0 = synth.se3(synth.rodrigues(np.array([0.1, -0.3, 0.2])), np.array([120.0, -40.0, 900.0]))
    return np.ascontiguousarray(np.stack([T0 @ P for P in poses]).astype(np.float32))


@needs_ref
@pytest.mark.parametrize("add_identity,transpose,inverse", [(1, 1, 0), (0, 1, 0), (1, 0, 0), (0, 0, 1), (1, 1, 1)])
def test_trajectory_file_is_the_reference_file(tmp_path, add_identity, transpose, inverse):
    P = trajectory()
    ours, theirs = tmp_path / "ours.txt", tmp_path / "ref.txt"
    t = rg.Trajectory(add_identity=bool(add_identity))
    for T in P:
        t.add_pose(T)
    t.save(str(ours), transpose=transpose, inverse=inverse)
    RL.lib().ref_result_save(os.fsencode(str(theirs)), O.ptr(P), len(P), add_identity, transpose, inverse)
    a, b = ours.read_bytes(), theirs.read_bytes()
    assert a == b
    assert a.count(b"\n") == len(P) + add_identity


def test_trajectory_round_trip(tmp_path):
    P = trajectory()
    path = str(tmp_path / "traj.txt")
    t = rg.Trajectory(add_identity=False)
    for T in P:
        t.add_pose(T)
    t.save(path)
    Q = rg.load_trajectory(path)
    assert len(Q) == len(P)
    # canonized in float: relative to the first pose (rotation to 2e-6, translation
    # in mm to float rounding of ~1 m lever arms), written with 7 significant digits
    expect = np.linalg.inv(P[0].astype(np.float64)) @ P.astype(np.float64)
    np.testing.assert_allclose(Q[:, :3, :3], expect[:, :3, :3], rtol=0, atol=2e-6)
    np.testing.assert_allclose(Q[:, :3, 3], expect[:, :3, 3], rtol=0, atol=5e-4)
    np.testing.assert_allclose(Q[0], np.eye(4), atol=1e-6)
    # without the transpose the file holds the transposed rows; reading it the
    # same way gives the same poses
    path2 = str(tmp_path / "traj_t0.txt")
    t.save(path2, transpose=0)
    np.testing.assert_array_equal(rg.load_trajectory(path2, transpose=0), Q)


def write_modes(path):
    rows = [(1, "photometric", 246.02), (30, "photometric", 242.31), (60, "biobjective-lambda0.75", 241.2),
            (90, "geometric", 238.7), (120, "biobjective-lambda0.25", 234.5), (150, "biobjective-lambda1.00", 230.0)]
    with open(path, "w") as f:
        for fr, m, e in rows:
            f.write(f"{fr:04d} {m} {e:f}\n")
    return rows


@needs_ref
def test_mode_list_matches_reference(tmp_path):
    path = str(tmp_path / "modes.tst")
    write_modes(path)
    params = rg.load_track_params(path)
    assert [p[1] for p in params] == [rg.PHOTOMETRIC, rg.PHOTOMETRIC, rg.BIOBJECTIVE, rg.GEOMETRIC, rg.BIOBJECTIVE,
                                      rg.BIOBJECTIVE]
    assert params[2][2] == np.float32(0.75) and params[3][2] == 1.0 and params[0][2] == 0.0
    fr = np.zeros(1, np.int32)
    md = np.zeros(1, np.int32)
    la = np.zeros(1, np.float32)
    for key in [-5, 0, 1, 15, 16, 45, 46, 74, 75, 76, 105, 135, 300]:
        RL.lib().ref_track_params_get(os.fsencode(path), key, O.ptr(fr), O.ptr(md), O.ptr(la))
        mine = rg.track_params_for(params, key)
        assert (mine[0], mine[1], np.float32(mine[2])) == (int(fr[0]), int(md[0]), la[0]), key


@needs_ref
def test_reference_mode_file_if_present():
    ref = os.environ.get("RECON_REFERENCE") or os.path.join(os.path.dirname(ROOT), "reference")
    path = os.path.join(ref, "bin", "data", "best-method.tst")
    if not os.path.exists(path):
        pytest.skip("the reference's data files are not here")
    params = rg.load_track_params(path)
    assert len(params) > 10
    fr = np.zeros(1, np.int32)
    md = np.zeros(1, np.int32)
    la = np.zeros(1, np.float32)
    for key in range(0, params[-1][0] + 40, 7):
        RL.lib().ref_track_params_get(os.fsencode(path), key, O.ptr(fr), O.ptr(md), O.ptr(la))
        mine = rg.track_params_for(params, key)
        assert (mine[0], mine[1], np.float32(mine[2])) == (int(fr[0]), int(md[0]), la[0]), key


def test_mode_list_errors(tmp_path):
    path = str(tmp_path / "bad.tst")
    with open(path, "w") as f:
        f.write("0001 photometric 1.0\n0030 sideways 2.0\n")
    with pytest.raises(rg.ReconError, match="invalid mode"):
        rg.load_track_params(path)
    with pytest.raises(rg.ReconError):
        rg.load_track_params(str(tmp_path / "missing.tst"))
    assert rg.track_params_for([], 12)[1] == rg.GEOMETRIC
