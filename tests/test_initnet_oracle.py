"""The CPU oracle of the learned initialisation network (checker of the GPU kernels).

Its FP64 gradient is checked against central finite differences of its own
loss, for parameters of every layer; the coarse-image formula is checked on
constant images.
"""
import ctypes

import numpy as np

import oracle_lib as O
from oracle_lib import ptr as p

LAYERS = [(4, 16), (16, 32), (32, 64), (64, 64), (64, 128), (128, 128)]


def _layout():
    off, q = [], 0
    for cin, cout in LAYERS:
        kp = (9 * cin + 15) // 16 * 16
        off.append((q, q + cout * kp, cin, cout, kp))
        q += cout * kp + cout
    return off, q, q + 6 * 128, q + 6 * 128 + 6 + 6  # ..., wfc, bfc, total (after the 6 output scales)


def _bf16(x):
    u = np.asarray(x, np.float32).view(np.uint32).astype(np.uint64)
    return ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint16)


def _problem(seed, n=2):
    rng = np.random.default_rng(seed)
    L = O.lib()
    total = int(L.orc_net_param_count())
    off, wfc, bfc, _ = _layout()
    params = np.zeros(total, np.float32)
    for w, b, cin, cout, kp in off:
        W = np.zeros((cout, kp), np.float32)
        W[:, : 9 * cin] = rng.normal(0, np.sqrt(2.0 / (9 * cin)), size=(cout, 9 * cin))
        params[w: w + cout * kp] = W.reshape(-1)
        params[b: b + cout] = rng.normal(0, 0.05, size=cout)
    params[wfc: wfc + 768] = rng.normal(0, 0.1, size=768)
    params[bfc: bfc + 6] = rng.normal(0, 0.1, size=6)
    inp = _bf16(rng.uniform(0, 1, size=(n, 60, 80, 4)))
    target = rng.normal(size=(n, 6)).astype(np.float32)
    return params, inp, target


def test_param_count_matches_layout():
    assert int(O.lib().orc_net_param_count()) == _layout()[3]


def test_gradient_matches_finite_differences():
    params, inp, target = _problem(1)
    L = O.lib()
    n = inp.shape[0]
    grad = np.zeros(params.size, np.float64)
    L.orc_net_loss_grad(p(params), p(inp), p(target), n, 1, p(grad))
    off, wfc, bfc, _ = _layout()
    rng = np.random.default_rng(2)
    picks = []
    for w, b, cin, cout, kp in off:
        co = rng.integers(0, cout, size=3)
        k = rng.integers(0, 9 * cin, size=3)
        picks += list(w + co * kp + k) + [b + int(rng.integers(0, cout))]
    picks += [wfc + 5, wfc + 300, bfc + 2]
    for i in picks:
        h = 1e-5 * max(abs(float(params[i])), 1e-2)  # small: ReLU kinks make the loss piecewise smooth
        pp = params.astype(np.float64)
        # the oracle takes FP32 parameters; exact mode evaluates in FP64, so
        # perturb by a step that FP32 represents exactly
        up = params.copy()
        dn = params.copy()
        up[i] = np.float32(pp[i] + h)
        dn[i] = np.float32(pp[i] - h)
        hh = (float(up[i]) - float(dn[i])) / 2
        g_tmp = np.zeros(params.size, np.float64)
        lu = L.orc_net_loss_grad(p(up), p(inp), p(target), n, 1, p(g_tmp))
        ld = L.orc_net_loss_grad(p(dn), p(inp), p(target), n, 1, p(g_tmp))
        fd = (lu - ld) / (2 * hh)
        assert abs(fd - grad[i]) <= 1e-3 * max(abs(grad[i]), 1e-3), (i, fd, grad[i])


def test_rounded_gradient_close_to_exact():
    params, inp, target = _problem(3)
    L = O.lib()
    g1 = np.zeros(params.size)
    g0 = np.zeros(params.size)
    L.orc_net_loss_grad(p(params), p(inp), p(target), 2, 1, p(g1))
    L.orc_net_loss_grad(p(params), p(inp), p(target), 2, 0, p(g0))
    assert np.linalg.norm(g0 - g1) <= 0.05 * np.linalg.norm(g1)


def test_coarse_of_constant_frames():
    W, H = 160, 120
    gray = np.full((1, H, W), 51, np.uint8)
    depth = np.full((1, H, W), 2000, np.uint16)
    depth[0, 0, 0] = 0  # an invalid pixel is left out of its block's depth mean
    depth[0, 2:4, 2:4] = 0  # a block without valid depth gives 0
    out = np.zeros((1, 60, 80, 2), np.uint16)
    O.lib().orc_net_coarse(p(gray), p(depth), 1, W, H, p(out))
    f = (out.astype(np.uint32) << 16).view(np.float32)
    assert np.allclose(f[..., 0], 0.2, atol=2e-3)
    assert f[0, 1, 1, 1] == 0.0
    f[0, 1, 1, 1] = 0.5
    assert np.allclose(f[..., 1], 0.5, atol=2e-3)
