"""GPU kernels of the learned initialisation network against the CPU oracle.

The forward pass (BF16 tensor-core convolutions, FP32 accumulation) and the
backward pass are compared with the oracle evaluated with the same BF16
rounding of weights and activations: they differ only by FP32 accumulation
order, which the tolerances below bound (relative L2 error per parameter
block).  The coarse-image kernel is integer plus a fixed sequence of FP32
operations and must match bit for bit.
"""
import numpy as np
import pytest

import oracle_lib as O
from oracle_lib import ptr as p

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

import recon_gb300.initnet as IN  # noqa: E402

# tolerances: FP32 accumulation-order differences, amplified where a BF16
# rounding of an activation flips
FWD_RTOL = 1e-2
GRAD_RTOL = 3e-2


def _need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _problem(seed, n):
    rng = np.random.default_rng(seed)
    params = IN.init_params(seed)
    off, wfc, bfc, sc, total = IN.layout()
    for (w, b), (cin, cout) in zip(off, IN.LAYERS):
        params[b: b + cout] = rng.normal(0, 0.05, size=cout)
    params[bfc: bfc + 6] = rng.normal(0, 0.1, size=6)
    x = rng.uniform(0, 1, size=(n, 60, 80, 4)).astype(np.float32)
    xb = torch.from_numpy(x).to(torch.bfloat16)
    inp_np = xb.view(torch.int16).numpy().view(np.uint16).copy()
    target = rng.normal(size=(n, 6)).astype(np.float32)
    return params, xb.cuda().contiguous(), inp_np, target


def _blocks():
    off, wfc, bfc, sc, total = IN.layout()
    out = []
    for l, ((w, b), (cin, cout)) in enumerate(zip(off, IN.LAYERS)):
        out.append((f"w{l}", w, b))
        out.append((f"b{l}", b, b + cout))
    out.append(("wfc", wfc, bfc))
    out.append(("bfc", bfc, sc))
    return out


def test_coarse_matches_oracle_bit_for_bit():
    _need_gpu()
    rng = np.random.default_rng(4)
    n, H, W = 3, 480, 640
    gray = rng.integers(0, 256, size=(n, H, W), dtype=np.uint8)
    depth = rng.integers(0, 4000, size=(n, H, W)).astype(np.uint16)
    depth[rng.uniform(size=depth.shape) < 0.2] = 0
    depth[1, :16, :16] = 0
    got = IN.coarse(torch.from_numpy(gray).cuda(), torch.from_numpy(depth.view(np.int16)).cuda())
    want = np.zeros((n, 60, 80, 2), np.uint16)
    O.lib().orc_net_coarse(p(gray), p(depth), n, W, H, p(want))
    assert np.array_equal(got.view(torch.int16).cpu().numpy().view(np.uint16), want)


def test_forward_matches_oracle():
    _need_gpu()
    n = 4
    params, inp, inp_np, _ = _problem(7, n)
    net = IN.InitNet(max_batch=8)
    net.set_params(params)
    y = net.forward(inp).cpu().numpy().astype(np.float64)
    want = np.zeros((n, 6))
    O.lib().orc_net_forward(p(params), p(inp_np), n, 0, p(want))
    assert np.linalg.norm(y - want) <= FWD_RTOL * np.linalg.norm(want), (y, want)


def test_gradient_matches_oracle_per_block():
    _need_gpu()
    n = 4
    params, inp, inp_np, target = _problem(8, n)
    net = IN.InitNet(max_batch=8)
    net.set_params(params)
    g, loss = net.gradient(inp, torch.from_numpy(target).cuda())
    g = g.cpu().numpy().astype(np.float64)
    want = np.zeros(params.size)
    lw = O.lib().orc_net_loss_grad(p(params), p(inp_np), p(target), n, 0, p(want))
    assert abs(float(loss.item()) - lw) <= 1e-3 * lw
    for name, a, b in _blocks():
        err = np.linalg.norm(g[a:b] - want[a:b])
        ref = np.linalg.norm(want[a:b])
        assert err <= GRAD_RTOL * ref + 1e-9, (name, err, ref)
    off, wfc, bfc, sc, total = IN.layout()
    assert np.all(g[sc:] == 0)


def test_large_batch_matches_oracle():
    """A batch of 64: the layer-1 forward runs pixel-parallel (at least 4096
    tiles of 16 output pixels), the input gradients of layers 1-2 reduce in
    one warp per row tile or split over two, and the layer-0 weight gradient
    adds 600 pixel splits by warps -- paths a batch of 4 does not take."""
    _need_gpu()
    n = 64
    params, inp, inp_np, target = _problem(11, n)
    net = IN.InitNet(max_batch=n)
    net.set_params(params)
    y = net.forward(inp).cpu().numpy().astype(np.float64)
    want = np.zeros((n, 6))
    O.lib().orc_net_forward(p(params), p(inp_np), n, 0, p(want))
    assert np.linalg.norm(y - want) <= FWD_RTOL * np.linalg.norm(want)
    g, loss = net.gradient(inp, torch.from_numpy(target).cuda())
    g = g.cpu().numpy().astype(np.float64)
    wg = np.zeros(params.size)
    lw = O.lib().orc_net_loss_grad(p(params), p(inp_np), p(target), n, 0, p(wg))
    assert abs(float(loss.item()) - lw) <= 1e-3 * lw
    for name, a, b in _blocks():
        err = np.linalg.norm(g[a:b] - wg[a:b])
        ref = np.linalg.norm(wg[a:b])
        assert err <= GRAD_RTOL * ref + 1e-9, (name, err, ref)


def test_gradient_is_deterministic():
    _need_gpu()
    params, inp, _, target = _problem(9, 16)
    net = IN.InitNet(max_batch=16)
    net.set_params(params)
    t = torch.from_numpy(target).cuda()
    g1, _ = net.gradient(inp, t)
    g2, _ = net.gradient(inp, t)
    assert torch.equal(g1, g2)


def test_adam_memorises_a_batch():
    _need_gpu()
    params, inp, _, target = _problem(10, 32)
    net = IN.InitNet(max_batch=32)
    net.set_params(params)
    t = torch.from_numpy(target).cuda()
    loss = torch.zeros(1, device="cuda")
    net.train_step(inp, t, 1e-3, loss)
    first = float(loss.item())
    for _ in range(300):
        net.train_step(inp, t, 1e-3, loss)
    assert float(loss.item()) < 0.05 * first
