"""GPU parity: librecon_track.so against the CPU oracle on the same inputs.

Integer outputs (masks, histograms, selected indices, ICP correspondence counts)
must be identical; the FP32/FP64 values are also required to be bit-identical,
because the kernels evaluate the reference's expressions in the same order
without FMA contraction and reduce the normal equations in the same canonical
order as the oracle.  The tolerance the tracking contract states (residuals
1e-5 relative, poses 1e-6 rad / 1e-6 m) is therefore met with zero error.
"""
import numpy as np
import pytest

import oracle_lib as O
import recon_gb300 as rg
from scenes import frame_pair, n_select_for

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def bits(a):
    a = np.ascontiguousarray(a)
    return a.view(np.uint32) if a.dtype == np.float32 else (a.view(np.uint64) if a.dtype == np.float64 else a)


def assert_bitexact(a, b, what):
    a = np.asarray(a)
    b = np.asarray(b)
    assert a.shape == b.shape, what
    if not np.array_equal(bits(a), bits(b)):
        diff = np.flatnonzero(bits(a).reshape(-1) != bits(b).reshape(-1))
        i = diff[0]
        raise AssertionError(f"{what}: {diff.size} of {a.size} differ; first at {i}: "
                             f"{a.reshape(-1)[i]!r} vs {b.reshape(-1)[i]!r}")


@pytest.fixture(scope="module", autouse=True)
def cuda_lib():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    rg.lib()


def run_pair(pair, mode, solver=rg.SOLVER_CHOLESKY, iters=None, n_select=None, lam=0.5, hist_bins=64):
    W, H, L = pair.W, pair.H, pair.L
    P = n_select or n_select_for(W, H)
    it = iters or (1, 3, 10, 5)
    cfg = rg.make_config(W, H, L, mode=mode, iters=it, n_select=P, solver=solver, lam=lam, hist_bins=hist_bins)
    trk = rg.Tracker(cfg, pair.cal.calib)
    trk.enable_trace(64)
    trk.set_reference(pair.g0, pair.d0)
    trk.set_current(pair.g1, pair.d1)
    T, st = trk.track()
    ocfg = O.make_config(W, H, L, mode=mode, iters=it, n_select=P, solver=solver, lam=lam, hist_bins=hist_bins)
    orc = O.OracleTracker(ocfg, pair.cal.calib)
    orc.set_reference(pair.g0, pair.d0)
    orc.set_current(pair.g1, pair.d1)
    To, tro = orc.track()
    return trk, orc, T, st, To, tro


CASES = [
    ("320x240", dict(W=320, H=240)),
    ("640x480_kc", dict(W=640, H=480, distortion=True)),
    ("160x120", dict(W=160, H=120)),
    ("80x60", dict(W=80, H=60)),
]


@pytest.fixture(scope="module", params=CASES, ids=[c[0] for c in CASES])
def pair(request):
    return frame_pair(**request.param[1])


def test_render_matches_cpu_twin():
    from recon_gb300 import synth
    cal = synth.make_calibration(640, 480, distortion=True)
    sc = synth.make_scene(3)
    T = synth.offset_pose(1, 5.0, 40.0)
    cam_ir = synth.camera_struct(cal, "L", T)
    cam_rgb = synth.camera_struct(cal, "R", T)
    g_cpu, d_cpu = O.render_pair(sc, cam_ir, cam_rgb, noise_rel=0.01, noise_seed=9, frame=4)
    d = torch.zeros((480, 640), dtype=torch.int16, device="cuda")
    g = torch.zeros((480, 640), dtype=torch.uint8, device="cuda")
    rg.render_depth(sc, cam_ir, 0.01, 9, 4, d)
    rg.render_gray(sc, cam_rgb, g)
    torch.cuda.synchronize()
    assert_bitexact(d.cpu().numpy().view(np.uint16), d_cpu, "depth")
    assert_bitexact(g.cpu().numpy(), g_cpu, "gray")


def test_reference_and_current_preparation(pair):
    W, H, L = pair.W, pair.H, pair.L
    P = n_select_for(W, H)
    trk, orc, *_ = run_pair(pair, rg.BIOBJECTIVE)
    for l in range(L):
        n = (W >> l) * (H >> l)
        assert_bitexact(trk.get_array(0, "ref_gray", l, np.float32, n), orc.get("ref_gray", l, n, np.float32),
                        f"ref gray L{l}")
        assert_bitexact(trk.get_array(0, "cur_gray", l, np.float32, n), orc.get("cur_gray", l, n, np.float32),
                        f"cur gray L{l}")
        rp = trk.get_array(0, "ref_pts", l, np.float32, 4 * n).reshape(n, 4)
        rn = trk.get_array(0, "ref_nrm", l, np.float32, 4 * n).reshape(n, 4)
        o6 = orc.get("ref6", l, 6 * n, np.float32).reshape(n, 6)
        om = orc.get("refmask", l, n, np.int32)
        assert_bitexact((rp[:, 3] != 0).astype(np.int32), om, f"ref mask L{l}")
        assert_bitexact(rp[:, :3], o6[:, :3], f"ref xyz L{l}")
        valid = om != 0
        assert_bitexact(rn[valid, :3], o6[valid, 3:6], f"ref normals L{l}")
        cp = trk.get_array(0, "cur_pts", l, np.float32, 4 * n).reshape(n, 4)
        c6 = orc.get("cur6", l, 6 * n, np.float32).reshape(n, 6)
        cm = orc.get("curmask", l, n, np.int32)
        assert_bitexact((cp[:, 3] != 0).astype(np.int32), cm, f"cur mask L{l}")
        assert_bitexact(cp[:, :3], c6[:, :3], f"cur xyz L{l}")
    assert_bitexact(trk.get_array(0, "sel_idx", 0, np.int32, P), orc.get("sel_idx", 0, P, np.int32), "selection")
    assert_bitexact(trk.get_array(0, "sel_xyz", 0, np.float32, 3 * P), orc.get("sel_xyz", 0, 3 * P, np.float32),
                    "selected xyz")
    for l in range(L):
        assert_bitexact(trk.get_array(0, "sel_I", l, np.float32, P), orc.get("sel_I", l, P, np.float32),
                        f"I_ref L{l}")
        assert_bitexact(trk.get_array(0, "sel_J", l, np.float32, 6 * P), orc.get("sel_J", l, 6 * P, np.float32),
                        f"J L{l}")


def compare_traces(tr_gpu, tr_orc):
    assert len(tr_gpu) == len(tr_orc)
    for k, (g, o) in enumerate(zip(tr_gpu, tr_orc)):
        where = f"iteration {k} (level {o.level}, iter {o.iter})"
        assert (g.level, g.iter, g.solved, g.icp_selected) == (o.level, o.iter, o.solved, o.icp_selected), where
        if o.median_bin >= 0:
            assert g.median_bin == o.median_bin, where
            assert_bitexact(np.array(g.hist), np.array(o.hist), "histogram " + where)
        assert_bitexact(np.array(g.A_ph), np.array(o.A_ph), "A_photo " + where)
        assert_bitexact(np.array(g.b_ph), np.array(o.b_ph), "b_photo " + where)
        assert_bitexact(np.array(g.A_icp), np.array(o.A_icp), "A_icp " + where)
        assert_bitexact(np.array(g.b_icp), np.array(o.b_icp), "b_icp " + where)
        assert_bitexact(np.array(g.T), np.array(o.T), "pose " + where)


@pytest.mark.parametrize("mode", [rg.PHOTOMETRIC, rg.GEOMETRIC, rg.BIOBJECTIVE], ids=["photo", "icp", "biobj"])
def test_tracking_trace_matches_oracle(pair, mode):
    trk, orc, T, st, To, tro = run_pair(pair, mode)
    compare_traces(trk.trace(0), tro)
    assert_bitexact(T, To, "final pose")
    assert st.iterations == len(tro)


def test_icp_correspondences_and_student_t_weights(pair):
    """The finest level's correspondence mask (icpResidualKernel2) and the final
    Student-t weights of every pixel (generateStudentTWeights), 0 where the pixel
    is not a correspondence."""
    trk, orc, T, st, To, tro = run_pair(pair, rg.BIOBJECTIVE)
    n = pair.W * pair.H
    mask = trk.get_array(0, "icp_mask", 0, np.uint8, n)
    sel = orc.get("icp_select", 0, n, np.int32)
    assert np.array_equal(np.flatnonzero(mask), sel), "correspondence mask"
    assert st.icp_selected[0] == sel.size
    assert_bitexact(trk.get_array(0, "icp_w", 0, np.float32, n), orc.get("icp_w_px", 0, n, np.float32),
                    "Student-t weights per pixel")


@pytest.mark.parametrize("iters", [(3, 0), (2, 2)], ids=["level1_only", "both_levels"])
def test_odd_level_size_matches_oracle(iters):
    """482x362 with two levels: level 1 is 241x181 = 43,621 pixels, not a
    multiple of 4 and above the fused preparation's limit, so its Student-t
    passes take the scalar loop instead of the four-pixel vector loads (level 0
    takes the vector loads).  With level 0 skipped, the per-pixel mask and
    weights left by level 1 are compared too."""
    p = frame_pair(482, 362, L=2, seed=31)
    trk, orc, T, st, To, tro = run_pair(p, rg.BIOBJECTIVE, iters=iters)
    compare_traces(trk.trace(0), tro)
    assert_bitexact(T, To, "final pose")
    if iters[1] == 0:
        n = (482 >> 1) * (362 >> 1)
        mask = trk.get_array(0, "icp_mask", 1, np.uint8, n)
        sel = orc.get("icp_select", 1, n, np.int32)
        assert np.array_equal(np.flatnonzero(mask), sel), "level-1 correspondence mask"
        assert_bitexact(trk.get_array(0, "icp_w", 1, np.float32, n), orc.get("icp_w_px", 1, n, np.float32),
                        "level-1 Student-t weights per pixel")


def test_cg_solver_matches_oracle():
    p = frame_pair(320, 240, seed=21)
    trk, orc, T, st, To, tro = run_pair(p, rg.BIOBJECTIVE, solver=rg.SOLVER_CG, iters=(10, 10, 10))
    compare_traces(trk.trace(0), tro)


def test_256_bin_mad_histogram():
    p = frame_pair(320, 240, seed=5)
    trk, orc, T, st, To, tro = run_pair(p, rg.PHOTOMETRIC, iters=(10, 10, 10), hist_bins=256)
    compare_traces(trk.trace(0), tro)


def test_batch_of_mixed_instances_matches_single_runs():
    pairs = [frame_pair(320, 240, seed=31), frame_pair(160, 120, seed=32), frame_pair(640, 480, seed=33),
             frame_pair(80, 60, seed=34)]
    modes = [rg.BIOBJECTIVE, rg.PHOTOMETRIC, rg.BIOBJECTIVE, rg.GEOMETRIC]
    iters = [(4, 6, 8), (3, 5, 7), (1, 3, 10, 5), (12, 4, 9)]
    cfgs = [rg.make_config(p.W, p.H, p.L, mode=m, iters=it, n_select=n_select_for(p.W, p.H))
            for p, m, it in zip(pairs, modes, iters)]
    b = rg.Batch(cfgs, [p.cal.calib for p in pairs])
    b.set_reference([p.g0 for p in pairs], [p.d0 for p in pairs])
    b.set_current([p.g1 for p in pairs], [p.d1 for p in pairs])
    T, st = b.track()
    for i, (p, m, it) in enumerate(zip(pairs, modes, iters)):
        ocfg = O.make_config(p.W, p.H, p.L, mode=m, iters=it, n_select=n_select_for(p.W, p.H))
        orc = O.OracleTracker(ocfg, p.cal.calib)
        orc.set_reference(p.g0, p.d0)
        orc.set_current(p.g1, p.d1)
        To, _ = orc.track()
        assert_bitexact(T[i], To, f"instance {i}")


def test_device_inputs_and_initial_pose():
    p = frame_pair(320, 240, seed=41)
    cfg = rg.make_config(320, 240, 3, mode=rg.BIOBJECTIVE, iters=(2, 3, 4))
    trk = rg.Tracker(cfg, p.cal.calib)
    g0 = torch.from_numpy(p.g0).cuda()
    d0 = torch.from_numpy(p.d0.view(np.int16)).cuda()
    g1 = torch.from_numpy(p.g1).cuda()
    d1 = torch.from_numpy(p.d1.view(np.int16)).cuda()
    trk.set_reference(g0, d0)
    trk.set_current(g1, d1)
    T0 = np.eye(4, dtype=np.float32)
    T0[:3, 3] = [3.0, -2.0, 5.0]
    T, st = trk.track(T0)
    ocfg = O.make_config(320, 240, 3, mode=rg.BIOBJECTIVE, iters=(2, 3, 4))
    orc = O.OracleTracker(ocfg, p.cal.calib)
    orc.set_reference(p.g0, p.d0)
    orc.set_current(p.g1, p.d1)
    To, _ = orc.track(T0)
    assert_bitexact(T, To, "pose from an initial guess")


def test_pose_accuracy_against_ground_truth():
    from recon_gb300 import synth
    p = frame_pair(640, 480, seed=51, noise=0.0)
    trk, orc, T, st, To, tro = run_pair(p, rg.BIOBJECTIVE)
    dt, dr = synth.pose_error(p.T_gt, T.astype(np.float64))
    assert dt < 1.0 and dr < 0.05, (dt, dr)


def _trajectory_frames(W, H, n, seed):
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
    return cal, poses, g, d


def test_sequence_tracking_matches_oracle():
    W, H = 320, 240
    cal, poses, g, d = _trajectory_frames(W, H, 6, seed=71)
    cfg = rg.make_config(W, H, 3, mode=rg.BIOBJECTIVE, iters=(2, 3, 4))
    b = rg.Batch([cfg], [cal.calib])
    b.set_reference([g[0]], [d[0]])
    T, st = b.track_sequence([[g[f]] for f in range(1, 6)], [[d[f]] for f in range(1, 6)])
    orc = O.OracleTracker(O.make_config(W, H, 3, mode=O.BIOBJECTIVE, iters=(2, 3, 4)), cal.calib)
    orc.set_reference(g[0], d[0])
    To = None
    for f in range(1, 6):
        orc.set_current(g[f], d[f])
        To, _ = orc.track(To)
        assert_bitexact(T[f - 1, 0], To, f"frame {f}")
    # host inputs (copied on the second stream) give the same poses
    b.set_reference([g[0]], [d[0]])
    T2, _ = b.track_sequence([[g[f]] for f in range(1, 6)], [[d[f]] for f in range(1, 6)])
    assert_bitexact(T2, T, "host vs device inputs")


def test_keyframe_fusion_matches_oracle():
    W, H = 320, 240
    cal, poses, g, d = _trajectory_frames(W, H, 8, seed=81)
    cfg = rg.make_config(W, H, 3, mode=rg.BIOBJECTIVE, iters=(2, 3, 4))
    b = rg.Batch([cfg], [cal.calib])
    b.set_reference([g[0]], [d[0]])
    T, _ = b.track_sequence([[g[f]] for f in range(1, 6)], [[d[f]] for f in range(1, 6)])
    b.fuse_keyframe([[d[f]] for f in range(1, 6)], T[:, :, :, :], gate_mm=30.0)
    T6, _ = b.track_sequence([[g[6]], [g[7]]], [[d[6]], [d[7]]])
    orc = O.OracleTracker(O.make_config(W, H, 3, mode=O.BIOBJECTIVE, iters=(2, 3, 4)), cal.calib)
    orc.set_reference(g[0], d[0])
    To, Ts = None, []
    for f in range(1, 6):
        orc.set_current(g[f], d[f])
        To, _ = orc.track(To)
        Ts.append(To.copy())
    orc.fuse_keyframe([d[f] for f in range(1, 6)], np.stack(Ts), gate=30.0)
    assert_bitexact(b.get_array(0, "ref_z", 0, np.float32, W * H), orc.get("ref_z", 0, W * H, np.float32),
                    "fused keyframe depth")
    P = 8192
    assert_bitexact(b.get_array(0, "sel_idx", 0, np.int32, P), orc.get("sel_idx", 0, P, np.int32),
                    "selection after fusion")
    for f in (6, 7):
        orc.set_current(g[f], d[f])
        To, _ = orc.track(To)
        assert_bitexact(T6[f - 6, 0], To, f"frame {f} after fusion")


def test_keyframe_rgbd_fusion_matches_oracle():
    """Depth and colour fusion of the frames of the tracked sequence with their
    poses, all taken on the device (no copy, no host round trip; here the
    library's device copies of host frames): the fused depth, the fused vertex
    colours, the rebuilt selection and intensities, and the poses of the
    frames tracked against the fused keyframe equal the oracle's."""
    W, H = 320, 240
    cal, poses, g, d = _trajectory_frames(W, H, 8, seed=83)
    cfg = rg.make_config(W, H, 3, mode=rg.BIOBJECTIVE, iters=(2, 3, 4))
    b = rg.Batch([cfg], [cal.calib])
    b.set_reference([g[0]], [d[0]])
    assert np.all(b.get_array(0, "ref_col", 0, np.float32, W * H) == -1.0), "a new keyframe has no fused colour"
    T, _ = b.track_sequence([[g[f]] for f in range(1, 6)], [[d[f]] for f in range(1, 6)])
    with pytest.raises(rg.ReconError):
        b.fuse_sequence(6)  # the sequence had five frames
    b.fuse_sequence(5, gate_mm=30.0)
    T6, _ = b.track_sequence([[g[6]], [g[7]]], [[d[6]], [d[7]]])
    orc = O.OracleTracker(O.make_config(W, H, 3, mode=O.BIOBJECTIVE, iters=(2, 3, 4)), cal.calib)
    orc.set_reference(g[0], d[0])
    To, Ts = None, []
    for f in range(1, 6):
        orc.set_current(g[f], d[f])
        To, _ = orc.track(To)
        Ts.append(To.copy())
    orc.fuse_keyframe([d[f] for f in range(1, 6)], np.stack(Ts), gate=30.0, grays=[g[f] for f in range(1, 6)])
    assert_bitexact(b.get_array(0, "ref_z", 0, np.float32, W * H), orc.get("ref_z", 0, W * H, np.float32),
                    "fused keyframe depth")
    col = b.get_array(0, "ref_col", 0, np.float32, W * H)
    assert_bitexact(col, orc.get("ref_col", 0, W * H, np.float32), "fused vertex colour")
    assert (col >= 0).mean() > 0.5, "most valid pixels have a fused colour"
    P = 8192
    assert_bitexact(b.get_array(0, "sel_idx", 0, np.int32, P), orc.get("sel_idx", 0, P, np.int32),
                    "selection after fusion")
    assert_bitexact(b.get_array(0, "sel_I", 0, np.float32, P), orc.get("sel_I", 0, P, np.float32),
                    "level-0 reference intensities (fused colours)")
    for f in (6, 7):
        orc.set_current(g[f], d[f])
        To, _ = orc.track(To)
        assert_bitexact(T6[f - 6, 0], To, f"frame {f} after fusion")
    # a new keyframe clears the fused colours
    b.set_reference([g[6]], [d[6]])
    assert np.all(b.get_array(0, "ref_col", 0, np.float32, W * H) == -1.0)
    # the caller's device frames give the same fused keyframe and poses
    gd = [torch.from_numpy(x).cuda() for x in g]
    dd = [torch.from_numpy(x.view(np.int16)).cuda() for x in d]
    b2 = rg.Batch([cfg], [cal.calib])
    b2.set_reference([gd[0]], [dd[0]])
    T2, _ = b2.track_sequence([[gd[f]] for f in range(1, 6)], [[dd[f]] for f in range(1, 6)])
    b2.fuse_sequence(5, gate_mm=30.0)
    T26, _ = b2.track_sequence([[gd[6]], [gd[7]]], [[dd[6]], [dd[7]]])
    assert_bitexact(b2.get_array(0, "ref_col", 0, np.float32, W * H), col, "fused colour, device frames")
    assert_bitexact(T26, T6, "poses after fusion, device frames")


def test_batch_with_uneven_resolutions_matches_oracle_per_iteration():
    """A batch whose launches are sized by its largest instance: every smaller
    instance must still match the oracle at every iteration (per-instance
    arrays indexed by block must not be touched by the extra blocks)."""
    specs = [(640, 480, 71), (320, 240, 72), (160, 120, 73), (80, 60, 74), (320, 240, 75), (160, 120, 76),
             (80, 60, 77), (320, 240, 78)]
    pairs = [frame_pair(w, h, seed=s, deg=3.0, mm=30.0) for w, h, s in specs]
    iters = [(4, 5, 6, 3), (5, 7, 4), (6, 4, 5), (7, 3, 6), (3, 6, 5), (4, 4, 4), (5, 5, 5), (6, 6, 2)]
    cfgs = [rg.make_config(p.W, p.H, p.L, mode=rg.BIOBJECTIVE, iters=it, n_select=n_select_for(p.W, p.H))
            for p, it in zip(pairs, iters)]
    b = rg.Batch(cfgs, [p.cal.calib for p in pairs])
    b.enable_trace(64)
    b.set_reference([p.g0 for p in pairs], [p.d0 for p in pairs])
    b.set_current([p.g1 for p in pairs], [p.d1 for p in pairs])
    for rep in range(2):
        T, _ = b.track(np.tile(np.eye(4, dtype=np.float32), (len(pairs), 1, 1)))
        for i, (p, it) in enumerate(zip(pairs, iters)):
            ocfg = O.make_config(p.W, p.H, p.L, mode=rg.BIOBJECTIVE, iters=it, n_select=n_select_for(p.W, p.H))
            orc = O.OracleTracker(ocfg, p.cal.calib)
            orc.set_reference(p.g0, p.d0)
            orc.set_current(p.g1, p.d1)
            To, tro = orc.track()
            compare_traces(b.trace(i), tro)
            assert_bitexact(T[i], To, f"instance {i} ({p.W}x{p.H}), run {rep}")
