"""Tracking with the learned initialisation against the oracle.

With a network attached, every frame's start pose comes from the gate between
the network's prediction and the previous pose.  The oracle is given the
network outputs the GPU produced (the network itself is checked separately
against its oracle, within FP32 accumulation tolerance) and must reproduce the
gate decisions and the tracked poses bit for bit, over a sequence, for a
network that predicts the true motion (the gate takes it) and for an untrained
one (the gate mostly falls back to the previous pose).
"""
import numpy as np
import pytest

import oracle_lib as O
import recon_gb300 as rg
from test_gpu_parity import _trajectory_frames, assert_bitexact

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

import recon_gb300.initnet as IN  # noqa: E402
from recon_gb300 import learn, synth  # noqa: E402

W, H, L = 320, 240, 3
ITERS = (1, 2, 2)


def _oracle_sequence(cal, g, d, outs, scale):
    orc = O.OracleTracker(O.make_config(W, H, L, mode=O.BIOBJECTIVE, iters=ITERS), cal.calib)
    orc.set_reference(g[0], d[0])
    T, ch = [], []
    for f in range(1, len(g)):
        orc.set_current(g[f], d[f])
        ch.append(orc.init_gate(outs[f - 1], scale))
        To, _ = orc.track(orc.pose())
        T.append(To.copy())
    return np.stack(T), np.array(ch)


def _run(params, cal, g, d, sequence_api):
    net = IN.InitNet(max_batch=4)
    net.set_params(params)
    cfg = rg.make_config(W, H, L, mode=rg.BIOBJECTIVE, iters=(2, 3, 4))
    b = rg.Batch([cfg], [cal.calib], stream=torch.cuda.current_stream().cuda_stream)
    b.set_init_net(net, ITERS)
    b.set_reference([g[0]], [d[0]])
    T, outs, ch = [], [], []
    if sequence_api:
        Ts, _ = b.track_sequence([[g[f]] for f in range(1, len(g))], [[d[f]] for f in range(1, len(g))])
        return Ts[:, 0], None, None, b
    for f in range(1, len(g)):
        b.set_current([g[f]], [d[f]])
        Tf, _ = b.track()
        c, o = b.init_choice()
        T.append(Tf[0].copy())
        outs.append(o[0].copy())
        ch.append(int(c[0]))
    return np.stack(T), np.stack(outs), np.array(ch), b


def _oracle_params(poses):
    """A network whose output is the true frame-to-frame twist of frame 1 (zero
    weights, bias = twist / scale)."""
    off, wfc, bfc, sc, total = IN.layout()
    p = np.zeros(total, np.float32)
    tw = learn.se3_log(synth.relative_pose(poses[0], poses[1])[None])[0]
    scale = np.full(6, 0.01, np.float32)
    p[bfc: bfc + 6] = (tw / scale).astype(np.float32)
    p[sc: sc + 6] = scale
    return p, scale


@pytest.mark.parametrize("kind", ["true_motion", "untrained"])
def test_learned_start_matches_oracle(kind):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    cal, poses, g, d = _trajectory_frames(W, H, 5, seed=91)
    if kind == "true_motion":
        params, scale = _oracle_params(poses)
    else:
        params = IN.init_params(3, np.full(6, 0.01, np.float32))
        scale = params[IN.layout()[3]: IN.layout()[3] + 6]
    T, outs, ch, _ = _run(params, cal, g, d, sequence_api=False)
    To, cho = _oracle_sequence(cal, g, d, outs, scale)
    assert np.array_equal(ch, cho), (ch, cho)
    assert_bitexact(T, To, f"learned-start poses ({kind})")
    if kind == "true_motion":
        assert ch[0] == 1  # the exact first motion beats the previous (identity) pose
    # the sequence entry point takes the same decisions and poses
    Ts, _, _, _ = _run(params, cal, g, d, sequence_api=True)
    assert_bitexact(Ts, T, f"sequence vs single-frame ({kind})")


def test_device_and_host_sequences_agree():
    """The sequence path with the network one frame ahead on a second stream:
    device-resident frames and host frames (staged one frame ahead) give the
    same decisions and poses, also for a second call on the same batch."""
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    cal, poses, g, d = _trajectory_frames(W, H, 6, seed=93)
    params = IN.init_params(5, np.full(6, 0.01, np.float32))
    out = []
    for on_device in (False, True):
        net = IN.InitNet(max_batch=2)
        net.set_params(params)
        cfg = rg.make_config(W, H, L, mode=rg.BIOBJECTIVE, iters=(2, 3, 4))
        b = rg.Batch([cfg, cfg], [cal.calib, cal.calib])
        b.set_init_net(net, ITERS)
        if on_device:
            gs = [torch.from_numpy(x).cuda() for x in g]
            ds = [torch.from_numpy(x.view(np.int16)).cuda() for x in d]
        else:
            gs, ds = g, d
        b.set_reference([gs[0], gs[1]], [ds[0], ds[1]])
        T1, _ = b.track_sequence([[gs[f], gs[f + 1]] for f in range(1, 4)], [[ds[f], ds[f + 1]] for f in range(1, 4)])
        T2, _ = b.track_sequence([[gs[f], gs[f]] for f in range(4, 6)], [[ds[f], ds[f]] for f in range(4, 6)])
        c, o = b.init_choice()
        out.append((T1, T2, c, o))
    for k, what in enumerate(("first call", "second call", "choices", "network outputs")):
        assert_bitexact(np.asarray(out[1][k]), np.asarray(out[0][k]), f"device vs host: {what}")


def test_detaching_restores_plain_tracking():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    cal, poses, g, d = _trajectory_frames(W, H, 3, seed=92)
    cfg = rg.make_config(W, H, L, mode=rg.BIOBJECTIVE, iters=(2, 3, 4))
    b = rg.Batch([cfg], [cal.calib])
    b.set_reference([g[0]], [d[0]])
    T0, _ = b.track_sequence([[g[1]], [g[2]]], [[d[1]], [d[2]]])
    net = IN.InitNet(max_batch=2)
    net.set_params(IN.init_params(1))
    b.set_init_net(net, ITERS)
    b.set_init_net(None)
    b.set_reference([g[0]], [d[0]])
    T1, _ = b.track_sequence([[g[1]], [g[2]]], [[d[1]], [d[2]]])
    assert_bitexact(T1, T0, "plain tracking after detaching the network")
