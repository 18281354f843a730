"""The learned initialisation network (include/recon_initnet.h) from Python.

A thin ctypes layer over librecon_track.so: the forward and backward passes,
Adam and the coarse-image preparation all run in the library's CUDA kernels;
tensors are torch CUDA tensors (BF16 inputs, FP32 targets and outputs).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import check, lib

NET_W, NET_H, NET_IN_CH, NET_OUT = 80, 60, 4, 6
LAYERS = [(4, 16), (16, 32), (32, 64), (64, 64), (64, 128), (128, 128)]
FEAT = 128


def _kpad(cin: int) -> int:
    return (9 * cin + 15) // 16 * 16


def layout():
    """Offsets of the flat parameter vector: per layer (w, b), then wfc, bfc, scale, total."""
    off, p = [], 0
    for cin, cout in LAYERS:
        w = p
        p += cout * _kpad(cin)
        b = p
        p += cout
        off.append((w, b))
    wfc = p
    p += NET_OUT * FEAT
    bfc = p
    p += NET_OUT
    scale = p
    p += NET_OUT
    return off, wfc, bfc, scale, p


def _lib():
    L = lib()
    if not getattr(L, "_initnet_bound", False):
        vp, i32 = ctypes.c_void_p, ctypes.c_int32
        L.recon_initnet_param_count.restype = ctypes.c_int64
        L.recon_initnet_create.argtypes = [i32, vp, ctypes.POINTER(vp)]
        L.recon_initnet_destroy.argtypes = [vp]
        L.recon_initnet_set_params.argtypes = [vp, vp, i32]
        L.recon_initnet_get_params.argtypes = [vp, vp]
        L.recon_initnet_forward.argtypes = [vp, vp, i32, vp]
        L.recon_initnet_gradient.argtypes = [vp, vp, vp, i32, vp, vp]
        L.recon_initnet_train_step.argtypes = [vp, vp, vp, i32, ctypes.c_float, vp]
        L.recon_initnet_coarse.argtypes = [vp, vp, i32, i32, i32, vp, vp]
        L.recon_initnet_pair.argtypes = [vp, vp, i32, vp, vp]
        L._initnet_bound = True
    return L


def param_count() -> int:
    return int(_lib().recon_initnet_param_count())


def init_params(seed: int, scale=None) -> np.ndarray:
    """He-normal convolution weights, zero biases, a small linear layer; `scale`
    (6 values, default 1) maps network outputs to the twist."""
    rng = np.random.default_rng(seed)
    off, wfc, bfc, sc, total = layout()
    p = np.zeros(total, np.float32)
    for (cin, cout), (w, _) in zip(LAYERS, off):
        kp = _kpad(cin)
        W = np.zeros((cout, kp), np.float32)
        W[:, : 9 * cin] = rng.normal(0.0, np.sqrt(2.0 / (9 * cin)), size=(cout, 9 * cin))
        p[w: w + cout * kp] = W.reshape(-1)
    p[wfc: wfc + NET_OUT * FEAT] = rng.normal(0.0, np.sqrt(1.0 / FEAT), size=NET_OUT * FEAT)
    p[sc: sc + NET_OUT] = 1.0 if scale is None else np.asarray(scale, np.float32)
    return p


class InitNet:
    def __init__(self, max_batch: int = 256, stream=None):
        """`stream`: the cudaStream_t all of the network's work runs on; by default
        torch's current stream (0 is the legacy default stream), so torch tensors
        passed in and out are ordered with it."""
        self.L = _lib()
        if stream is None:
            import torch
            stream = torch.cuda.current_stream().cuda_stream
        h = ctypes.c_void_p()
        check(self.L.recon_initnet_create(max_batch, ctypes.c_void_p(stream), ctypes.byref(h)))
        self.h = h
        self.max_batch = max_batch
        self.n_params = param_count()

    def close(self):
        if self.h:
            self.L.recon_initnet_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_params(self, params):
        if hasattr(params, "data_ptr"):
            check(self.L.recon_initnet_set_params(self.h, ctypes.c_void_p(params.data_ptr()), 1))
        else:
            p = np.ascontiguousarray(params, np.float32)
            check(self.L.recon_initnet_set_params(self.h, p.ctypes.data_as(ctypes.c_void_p), 0))

    def get_params(self) -> np.ndarray:
        p = np.zeros(self.n_params, np.float32)
        check(self.L.recon_initnet_get_params(self.h, p.ctypes.data_as(ctypes.c_void_p)))
        return p

    def forward(self, inp, out=None):
        import torch
        n = inp.shape[0]
        if out is None:
            out = torch.empty((n, NET_OUT), dtype=torch.float32, device=inp.device)
        check(self.L.recon_initnet_forward(self.h, ctypes.c_void_p(inp.data_ptr()), n,
                                           ctypes.c_void_p(out.data_ptr())))
        return out

    def gradient(self, inp, target):
        import torch
        n = inp.shape[0]
        g = torch.empty(self.n_params, dtype=torch.float32, device=inp.device)
        loss = torch.empty(1, dtype=torch.float32, device=inp.device)
        check(self.L.recon_initnet_gradient(self.h, ctypes.c_void_p(inp.data_ptr()),
                                            ctypes.c_void_p(target.data_ptr()), n, ctypes.c_void_p(g.data_ptr()),
                                            ctypes.c_void_p(loss.data_ptr())))
        return g, loss

    def train_step(self, inp, target, lr: float, loss_out):
        check(self.L.recon_initnet_train_step(self.h, ctypes.c_void_p(inp.data_ptr()),
                                              ctypes.c_void_p(target.data_ptr()), inp.shape[0], float(lr),
                                              ctypes.c_void_p(loss_out.data_ptr())))


def coarse(gray, depth, stream=None):
    """[n, H, W] uint8 gray and int16/uint16 depth (CUDA) -> [n, 60, 80, 2] BF16 coarse images."""
    import torch
    n, H, W = gray.shape
    out = torch.empty((n, NET_H, NET_W, 2), dtype=torch.bfloat16, device=gray.device)
    check(_lib().recon_initnet_coarse(ctypes.c_void_p(gray.data_ptr()), ctypes.c_void_p(depth.data_ptr()), n, W, H,
                                      ctypes.c_void_p(out.data_ptr()), stream))
    return out


def pair(prev, cur, stream=None):
    """Network inputs [n, 60, 80, 4] from coarse images of the previous and current frames."""
    import torch
    n = prev.shape[0]
    out = torch.empty((n, NET_H, NET_W, NET_IN_CH), dtype=torch.bfloat16, device=prev.device)
    check(_lib().recon_initnet_pair(ctypes.c_void_p(prev.data_ptr()), ctypes.c_void_p(cur.data_ptr()), n,
                                    ctypes.c_void_p(out.data_ptr()), stream))
    return out
