"""The settle rule: a pyramid level ends early once one Gauss-Newton iteration
has moved every translation entry of the pose by at most `settle_mm` and every
rotation entry by at most `settle_rot`; the level's iteration count stays the
cap.  The reference runs a fixed schedule (gpuEstimateIncrement,
phototracker.cpp:666-689); with the rule off (settle_mm 0, the default) the
tracker is that schedule.

CPU tests check the oracle's rule; the GPU tests check that librecon_track.so
takes the same decisions (poses and executed iterations bit-identical to the
oracle) with instances that settle and instances that do not sharing every
launch.
"""
import numpy as np
import pytest

import oracle_lib as O
from scenes import frame_pair


def _oracle_run(p, iters, settle, T0=None):
    cfg = O.make_config(p.W, p.H, p.L, mode=O.BIOBJECTIVE, iters=iters, settle=settle)
    orc = O.OracleTracker(cfg, p.cal.calib)
    orc.set_reference(p.g0, p.d0)
    orc.set_current(p.g1, p.d1)
    T, tr = orc.track(T0)
    orc.close()
    return T, tr


def test_settle_off_is_the_fixed_schedule():
    p = frame_pair(160, 120, seed=13)
    T0, tr0 = _oracle_run(p, (3, 4, 5), (0.0, 0.0))
    assert [t.level for t in tr0] == [2] * 3 + [1] * 4 + [0] * 5


def test_settle_ends_each_level_after_the_first_small_step():
    p = frame_pair(160, 120, seed=13)
    I = np.eye(4, dtype=np.float32)
    T_fix, tr_fix = _oracle_run(p, (3, 4, 5), (0.0, 0.0), I)
    # a huge tolerance: every level stops after its first iteration
    T_one, tr_one = _oracle_run(p, (3, 4, 5), (1e30, 1e30), I)
    assert [t.level for t in tr_one] == [2, 1, 0]
    T_sched, _ = _oracle_run(p, (1, 1, 1), (0.0, 0.0), I)
    assert np.array_equal(T_one.view(np.uint32), T_sched.view(np.uint32))
    # a finite tolerance: a level ends exactly after the first iteration whose
    # pose change is within it, or at its cap
    tol = (0.05, 5e-5)
    caps = {2: 3, 1: 4, 0: 5}
    T_s, tr_s = _oracle_run(p, (3, 4, 5), tol, I)
    assert len(tr_s) < len(tr_fix)
    prev = I.reshape(16).copy()
    for k, t in enumerate(tr_s):
        cur = np.array(t.T, np.float32)
        settled = O.lib().orc_pose_settled(O.ptr(prev), O.ptr(cur), np.float32(tol[0]), np.float32(tol[1]))
        last_of_level = k + 1 == len(tr_s) or tr_s[k + 1].level != t.level
        assert last_of_level == (bool(settled) or t.iter + 1 == caps[t.level]), k
        prev = cur
    # up to the first early exit the run is the fixed schedule's
    first = next((i for i, (a, b) in enumerate(zip(tr_s, tr_fix)) if a.level != b.level), len(tr_s))
    for i in range(first):
        assert np.array_equal(np.array(tr_s[i].T, np.float32).view(np.uint32),
                              np.array(tr_fix[i].T, np.float32).view(np.uint32))


def test_pose_settled_comparisons():
    L = O.lib()
    a = np.eye(4, dtype=np.float32).reshape(16)
    b = a.copy()
    f = np.float32
    assert L.orc_pose_settled(O.ptr(a), O.ptr(b), f(0.0), f(0.0)) == 1  # no change settles at tolerance 0
    b[3] = 0.5  # translation x
    assert L.orc_pose_settled(O.ptr(a), O.ptr(b), f(0.5), f(0.0)) == 1
    assert L.orc_pose_settled(O.ptr(a), O.ptr(b), f(0.4999), f(1.0)) == 0
    b[3] = 0.0
    b[1] = 1e-4  # rotation entry
    assert L.orc_pose_settled(O.ptr(a), O.ptr(b), f(1.0), f(1e-4)) == 1
    assert L.orc_pose_settled(O.ptr(a), O.ptr(b), f(1.0), f(9e-5)) == 0
    b[1] = np.nan
    assert L.orc_pose_settled(O.ptr(a), O.ptr(b), f(1e30), f(1e30)) == 0
    b[1] = 0.0
    b[12] = 7.0  # the bottom row is not compared
    assert L.orc_pose_settled(O.ptr(a), O.ptr(b), f(0.0), f(0.0)) == 1


# ---------------------------------------------------------------- GPU
def _trajectory(W, H, n, seed):
    from recon_gb300 import synth
    cal = synth.make_calibration(W, H)
    sc = synth.make_scene(seed)
    poses = synth.smooth_trajectory(n, seed + 2, max_step_mm=10.0, max_step_deg=0.7)
    g, d = [], []
    for f in range(n):
        gf, df = O.render_pair(sc, synth.camera_struct(cal, "L", poses[f]), synth.camera_struct(cal, "R", poses[f]),
                               noise_rel=0.01, noise_seed=seed + 1, frame=f)
        g.append(gf)
        d.append(df)
    return cal, g, d


# (mode, iteration caps, settle tolerances) of the instances of one batch
GPU_INSTANCES = [
    (O.BIOBJECTIVE, (3, 6, 8), (0.05, 5e-5)),
    (O.BIOBJECTIVE, (3, 6, 8), (0.0, 0.0)),
    (O.PHOTOMETRIC, (4, 6, 8), (0.2, 2e-4)),
    (O.GEOMETRIC, (3, 5, 6), (0.02, 2e-5)),
]


@pytest.mark.gpu
def test_settle_rule_matches_oracle_in_shared_launches():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import recon_gb300 as rg
    W, H, nf = 320, 240, 6
    cal, g, d = _trajectory(W, H, nf, seed=61)
    cfgs = [rg.make_config(W, H, 3, mode=m, iters=it) for m, it, _ in GPU_INSTANCES]
    n = len(cfgs)
    b = rg.Batch(cfgs, [cal.calib] * n)
    for i, (_, _, s) in enumerate(GPU_INSTANCES):
        b.set_settle(i, *s)
    b.set_reference([g[0]] * n, [d[0]] * n)
    orcs = []
    for m, it, s in GPU_INSTANCES:
        o = O.OracleTracker(O.make_config(W, H, 3, mode=m, iters=it, settle=s), cal.calib)
        o.set_reference(g[0], d[0])
        orcs.append(o)
    T = np.tile(np.eye(4, dtype=np.float32), (n, 1, 1))
    To = [None] * n
    fired = 0
    for f in range(1, nf):
        b.set_current([g[f]] * n, [d[f]] * n)
        T, st = b.track(T)
        for i, o in enumerate(orcs):
            o.set_current(g[f], d[f])
            To[i], tr = o.track(To[i])
            assert np.array_equal(T[i].view(np.uint32), To[i].view(np.uint32)), (f, i)
            assert st[i].iterations == len(tr), (f, i, st[i].iterations, len(tr))
            if GPU_INSTANCES[i][2][0] > 0:
                fired += sum(GPU_INSTANCES[i][1]) - len(tr)
            else:
                assert len(tr) == sum(GPU_INSTANCES[i][1])
    assert fired > 0  # the rule skipped iterations
    # switching the rule off restores the fixed schedule (same launches)
    for i in range(n):
        b.set_settle(i, 0.0, 0.0)
    b.set_current([g[1]] * n, [d[1]] * n)
    T1, st1 = b.track()
    for i in range(n):
        assert st1[i].iterations == sum(GPU_INSTANCES[i][1])
    for o in orcs:
        o.close()
    b.close()


@pytest.mark.gpu
def test_settle_rule_in_graph_replayed_sequences():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import recon_gb300 as rg
    W, H, nf = 320, 240, 6
    cal, g, d = _trajectory(W, H, nf, seed=67)
    m, it, s = GPU_INSTANCES[0]
    cfg = rg.make_config(W, H, 3, mode=m, iters=it, settle=s)
    b = rg.Batch([cfg, cfg], [cal.calib] * 2)
    b.set_settle(1, 0.0, 0.0)
    b.set_reference([g[0]] * 2, [d[0]] * 2)
    T, _ = b.track_sequence([[g[f]] * 2 for f in range(1, nf)], [[d[f]] * 2 for f in range(1, nf)])
    for inst, settle in ((0, s), (1, (0.0, 0.0))):
        o = O.OracleTracker(O.make_config(W, H, 3, mode=m, iters=it, settle=settle), cal.calib)
        o.set_reference(g[0], d[0])
        To = None
        for f in range(1, nf):
            o.set_current(g[f], d[f])
            To, _ = o.track(To)
            assert np.array_equal(T[f - 1, inst].view(np.uint32), To.view(np.uint32)), (inst, f)
        o.close()
    b.close()


@pytest.mark.gpu
def test_settle_rule_through_the_tracker_entry_points():
    """recon_tracker_create with a settle configuration, and recon_set_settle
    switching it off and on again: poses and executed iterations equal the
    oracle's with the same rule."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import ctypes
    import recon_gb300 as rg
    p = frame_pair(320, 240, seed=29)
    iters, tol = (3, 6, 8), (0.05, 5e-5)
    trk = rg.Tracker(rg.make_config(320, 240, 3, mode=rg.BIOBJECTIVE, iters=iters, settle=tol), p.cal.calib)
    trk.set_reference(p.g0, p.d0)
    trk.set_current(p.g1, p.d1)
    I = np.eye(4, dtype=np.float32)
    for settle in (tol, (0.0, 0.0), tol):
        rg.check(rg.lib().recon_set_settle(trk.h, ctypes.c_float(settle[0]), ctypes.c_float(settle[1])))
        T, st = trk.track(I)
        To, tr = _oracle_run(p, iters, settle, I)
        assert np.array_equal(np.asarray(T, np.float32).view(np.uint32), To.view(np.uint32)), settle
        assert st.iterations == len(tr), (settle, st.iterations, len(tr))
    assert len(_oracle_run(p, iters, tol, I)[1]) < sum(iters)
    # invalid tolerances are refused
    assert rg.lib().recon_set_settle(trk.h, ctypes.c_float(-1.0), ctypes.c_float(0.0)) < 0
    assert rg.lib().recon_set_settle(trk.h, ctypes.c_float(float("nan")), ctypes.c_float(0.0)) < 0
