"""The frame-stack form of the batch API (set_reference_frames,
set_current_frames, track_sequence_frames).

It builds the input pointer tables with numpy from one stack of frames and an
index array instead of one tensor view per frame; the C entry points and the
tracking are the list form's, so the poses must agree bit for bit.  The pointer
arithmetic and the argument checks are host logic and run without a GPU; the
agreement is checked on the GPU for device and pinned-host stacks, with and
without the learned start.
"""
import numpy as np
import pytest

import recon_gb300 as rg


def _host_batch(n, w, h):
    """A Batch with only the host-side fields the pointer tables read (no
    device handle: it is never passed to the library)."""
    b = object.__new__(rg.Batch)
    b.n, b.configs = n, [rg.make_config(w, h, 3)] * n
    b._resolutions = {(w, h)}
    return b


def test_stack_table_addresses_and_checks():
    fb = _host_batch(3, 64, 32)
    stack = np.zeros((5, 32, 64), np.uint8)
    idx = np.array([[0, 4, 2], [1, 1, 3]])
    table, dev = fb._stack_table(stack, idx, 1)
    assert dev == 0 and table.dtype == np.uint64 and table.shape == idx.shape
    assert table.flags["C_CONTIGUOUS"]
    for f in range(2):
        for i in range(3):
            assert int(table[f, i]) == stack[idx[f, i]].ctypes.data
    depth = np.zeros((5, 32, 64), np.uint16)
    table, _ = fb._stack_table(depth, idx, 2)
    assert int(table[1, 2]) == depth[3].ctypes.data
    with pytest.raises(IndexError):
        fb._stack_table(stack, np.array([5]), 1)
    with pytest.raises(IndexError):
        fb._stack_table(stack, np.array([-1]), 1)
    with pytest.raises(ValueError):  # element size
        fb._stack_table(depth, idx, 1)
    with pytest.raises(ValueError):  # resolution
        fb._stack_table(np.zeros((5, 64, 32), np.uint8), idx, 1)
    with pytest.raises(ValueError):  # not contiguous
        fb._stack_table(np.zeros((5, 32, 128), np.uint8)[:, :, ::2], idx, 1)
    with pytest.raises(ValueError):  # index shape
        fb._stack_tables(stack, depth, idx, (3,))
    torch = pytest.importorskip("torch")
    t = torch.zeros((5, 32, 64), dtype=torch.int16)
    table, dev = fb._stack_table(t, np.array([2]), 2)
    assert dev == 0 and int(table[0]) == t[2].data_ptr()


@pytest.mark.gpu
@pytest.mark.parametrize("learned", [False, True])
def test_frame_stacks_track_like_lists(learned):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from test_gpu_parity import _trajectory_frames, assert_bitexact
    import recon_gb300.initnet as IN
    W, H, L = 320, 240, 3
    cal, poses, g, d = _trajectory_frames(W, H, 7, seed=95)
    gd = torch.from_numpy(np.stack(g)).cuda()
    dd = torch.from_numpy(np.stack([x.view(np.int16) for x in d])).cuda()
    gh = torch.from_numpy(np.stack(g)).pin_memory().numpy()
    dh = torch.from_numpy(np.stack(d).view(np.int16)).pin_memory().numpy().view(np.uint16)
    ref = np.array([0, 1])
    seq = np.array([[f, f + 1] for f in range(1, 6)])

    def batch():
        cfg = rg.make_config(W, H, L, mode=rg.BIOBJECTIVE, iters=(2, 3, 4))
        b = rg.Batch([cfg, cfg], [cal.calib, cal.calib])
        if learned:
            net = IN.InitNet(max_batch=2)
            net.set_params(IN.init_params(5, np.full(6, 0.01, np.float32)))
            b.set_init_net(net, (1, 2, 2))
            b._net = net
        return b

    b = batch()
    b.set_reference([g[i] for i in ref], [d[i] for i in ref])
    T_list, _ = b.track_sequence([[g[i] for i in row] for row in seq], [[d[i] for i in row] for row in seq])
    for gs, ds, what in ((gd, dd, "device stack"), (gh, dh, "pinned host stack")):
        b = batch()
        b.set_reference_frames(gs, ds, ref)
        T, _ = b.track_sequence_frames(gs, ds, seq)
        assert_bitexact(T, T_list, f"{what} vs lists")
    # single-frame form
    b = batch()
    b.set_reference_frames(gd, dd, ref)
    b.set_current_frames(gd, dd, seq[0])
    T1, _ = b.track()
    b2 = batch()
    b2.set_reference([g[i] for i in ref], [d[i] for i in ref])
    b2.set_current([g[i] for i in seq[0]], [d[i] for i in seq[0]])
    T2, _ = b2.track()
    assert_bitexact(T1, T2, "set_current_frames vs set_current")


@pytest.mark.gpu
def test_host_stack_steps_with_fusion_match_device_stack():
    """Two steps of: keyframes, five tracked frames, their fusion into the
    keyframes, two more tracked frames -- from a pinned host stack (the
    library copies host frames into slot sets that alternate by call, so a
    call's copies overlap the fusion of the previous call's frames) and from
    the same frames on the device: poses and fused keyframes bit-identical."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from test_gpu_parity import _trajectory_frames, assert_bitexact
    W, H, L = 320, 240, 3
    cal, poses, g, d = _trajectory_frames(W, H, 9, seed=97)
    gd = torch.from_numpy(np.stack(g)).cuda()
    dd = torch.from_numpy(np.stack([x.view(np.int16) for x in d])).cuda()
    gh = torch.from_numpy(np.stack(g)).pin_memory().numpy()
    dh = torch.from_numpy(np.stack(d).view(np.int16)).pin_memory().numpy().view(np.uint16)
    ref = np.array([0, 1])
    seq1 = np.array([[f, f + 1] for f in range(1, 6)])
    seq2 = np.array([[6, 7], [7, 8]])
    out = {}
    for gs, ds, what in ((gd, dd, "device"), (gh, dh, "host")):
        cfg = rg.make_config(W, H, L, mode=rg.BIOBJECTIVE, iters=(2, 3, 4))
        b = rg.Batch([cfg, cfg], [cal.calib, cal.calib])
        res = []
        for _ in range(2):
            b.set_reference_frames(gs, ds, ref)
            T1, _ = b.track_sequence_frames(gs, ds, seq1)
            b.fuse_sequence(5, gate_mm=30.0)
            T2, _ = b.track_sequence_frames(gs, ds, seq2)
            res.append((T1, T2, b.get_array(1, "ref_z", 0, np.float32, W * H),
                        b.get_array(1, "ref_col", 0, np.float32, W * H)))
        out[what] = res
    for k in range(2):
        for a, c, name in zip(out["host"][k], out["device"][k], ("poses before", "poses after", "depth", "colour")):
            assert_bitexact(a, c, f"step {k}: {name} of the fusion, host vs device stack")
    assert_bitexact(out["host"][1][1], out["host"][0][1], "the second step repeats the first")
