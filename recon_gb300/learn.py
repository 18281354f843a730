"""Training data and training of the learned initialisation network.

Frame pairs come from seeded procedural scenes and smooth camera trajectories
(consecutive frames and frames up to `max_gap` apart), rendered at 640x480 by
the library's ray caster; each pair is labelled with the pose the plain tracker
converges to (BIOBJECTIVE, full schedule, started from the identity), and the
label is that pose's twist in the tracker's SE(3) convention.  The network is
trained on the GPU by the library's own forward / backward / Adam kernels.

Run as a module to train and save parameters:
    python -m recon_gb300.learn --pairs 200000 --epochs 10 --out <file.npz>
or to time the training step alone (random inputs, CUDA events):
    python -m recon_gb300.learn --time-steps 20 [--batch 256]
"""
from __future__ import annotations

import argparse
import math
import time

import numpy as np

from . import synth

W, H, LEVELS = 640, 480, 4
ITERS = (1, 3, 10, 5)
LAMBDA = 0.5
N_SELECT = 8192
SCALE_OUT = 1000.0  # translation scale of the tracker's pose update (mm per twist unit)


def se3_log(T: np.ndarray) -> np.ndarray:
    """Twists x [n, 6] with T = exp(A(x)) (translation times SCALE_OUT), for
    rotations below pi: A(x) = [[0, -x2, x1, x3], [x2, 0, -x0, x4], [-x1, x0, 0, x5], 0]."""
    T = np.asarray(T, np.float64).reshape(-1, 4, 4)
    R, t = T[:, :3, :3], T[:, :3, 3] / SCALE_OUT
    c = np.clip((np.trace(R, axis1=1, axis2=2) - 1.0) / 2.0, -1.0, 1.0)
    th = np.arccos(c)
    v = np.stack([R[:, 2, 1] - R[:, 1, 2], R[:, 0, 2] - R[:, 2, 0], R[:, 1, 0] - R[:, 0, 1]], axis=1)
    small = th < 1e-6
    f = np.where(small, 0.5 + th * th / 12.0, th / (2.0 * np.sin(np.where(small, 1.0, th))))
    w = v * f[:, None]
    Wm = np.zeros((len(T), 3, 3))
    Wm[:, 0, 1], Wm[:, 0, 2] = -w[:, 2], w[:, 1]
    Wm[:, 1, 0], Wm[:, 1, 2] = w[:, 2], -w[:, 0]
    Wm[:, 2, 0], Wm[:, 2, 1] = -w[:, 1], w[:, 0]
    th2 = np.where(small, 1.0, th * th)
    coef = np.where(small, 1.0 / 12.0,
                    (1.0 - (th * np.sin(th)) / (2.0 * (1.0 - np.cos(np.where(small, 1.0, th))))) / th2)
    I = np.eye(3)[None]
    Vinv = I - 0.5 * Wm + coef[:, None, None] * (Wm @ Wm)
    u = np.einsum("nij,nj->ni", Vinv, t)
    return np.concatenate([w, u], axis=1)


def se3_exp(x: np.ndarray) -> np.ndarray:
    """Inverse of se3_log (float64, [n, 6] -> [n, 4, 4])."""
    from scipy.linalg import expm
    x = np.asarray(x, np.float64).reshape(-1, 6)
    out = np.zeros((len(x), 4, 4))
    for i, v in enumerate(x):
        A = np.array([[0, -v[2], v[1], v[3]], [v[2], 0, -v[0], v[4]], [-v[1], v[0], 0, v[5]], [0, 0, 0, 0]])
        E = expm(A)
        E[:3, 3] *= SCALE_OUT
        out[i] = E
    return out


def make_pairs(n_pairs: int, seed: int, max_gap: int = 3, batch: int = 256, pairs_per_scene: int = 64,
               traj_len: int = 200, log=print):
    """Renders and labels n_pairs frame pairs.  Returns (inputs [n, 60, 80, 4]
    BF16 CUDA tensor, twists [n, 6] float32 numpy, ground-truth relative poses
    [n, 4, 4] float64 numpy).  Scene s uses seed `seed + s`."""
    import torch

    import recon_gb300 as rg

    from . import initnet as IN

    cal = synth.make_calibration(W, H)
    stream = torch.cuda.current_stream().cuda_stream
    cfg = rg.make_config(W, H, LEVELS, mode=rg.BIOBJECTIVE, iters=ITERS, n_select=N_SELECT, lam=LAMBDA)
    tracker = rg.Batch([cfg] * batch, [cal.calib] * batch, stream=stream)
    inputs = torch.empty((n_pairs, IN.NET_H, IN.NET_W, IN.NET_IN_CH), dtype=torch.bfloat16, device="cuda")
    twists = np.zeros((n_pairs, 6), np.float32)
    gt = np.zeros((n_pairs, 4, 4))
    g = torch.empty((2 * batch, H, W), dtype=torch.uint8, device="cuda")
    d = torch.empty((2 * batch, H, W), dtype=torch.int16, device="cuda")
    rng = np.random.default_rng(seed)
    t0 = time.time()
    done = 0
    scene_id = 0
    scene = traj = None
    left_in_scene = 0
    while done < n_pairs:
        nb = min(batch, n_pairs - done)
        rel = np.zeros((nb, 4, 4))
        for k in range(nb):
            if left_in_scene == 0:
                scene = synth.make_scene(seed + scene_id)
                traj = synth.smooth_trajectory(traj_len, seed + 7919 * (scene_id + 1))
                scene_id += 1
                left_in_scene = pairs_per_scene
            left_in_scene -= 1
            gap = int(rng.integers(1, max_gap + 1))
            f = int(rng.integers(0, traj_len - gap))
            fid = 2 * (done + k)
            for j, fr in enumerate((f, f + gap)):
                rg.render_depth(scene, synth.camera_struct(cal, "L", traj[fr]), 0.01, seed + 1, fid + j,
                                d[2 * k + j])
                rg.render_gray(scene, synth.camera_struct(cal, "R", traj[fr]), g[2 * k + j])
            rel[k] = synth.relative_pose(traj[f], traj[f + gap])
        refs = [g[2 * k] for k in range(nb)] + [g[0]] * (batch - nb)
        refd = [d[2 * k] for k in range(nb)] + [d[0]] * (batch - nb)
        curs = [g[2 * k + 1] for k in range(nb)] + [g[1]] * (batch - nb)
        curd = [d[2 * k + 1] for k in range(nb)] + [d[1]] * (batch - nb)
        tracker.set_reference(refs, refd)
        tracker.set_current(curs, curd)
        T, _ = tracker.track(np.tile(np.eye(4, dtype=np.float32), (batch, 1, 1)))
        co = IN.coarse(g[: 2 * nb], d[: 2 * nb])
        inputs[done: done + nb] = IN.pair(co[0::2].contiguous(), co[1::2].contiguous())
        twists[done: done + nb] = se3_log(T[:nb])
        gt[done: done + nb] = rel
        done += nb
        if log and (done // batch) % 50 == 0:
            log(f"pairs {done}/{n_pairs} ({time.time() - t0:.0f} s)")
    torch.cuda.synchronize()
    return inputs, twists, gt


def train(inputs, twists: np.ndarray, epochs: int, batch: int = 256, lr: float = 1e-3, seed: int = 0,
          log=print):
    """Adam on the normalised twists; returns (FP32 parameters, loss history)."""
    import torch

    from . import initnet as IN

    n = inputs.shape[0]
    scale = twists.std(axis=0).astype(np.float32) + 1e-6
    params = IN.init_params(seed, scale)
    net = IN.InitNet(max_batch=batch)
    net.set_params(params)
    tgt = torch.from_numpy(twists / scale).float().cuda()
    gen = torch.Generator(device="cpu")
    gen.manual_seed(seed)
    loss = torch.zeros(1, device="cuda")
    steps = epochs * (n // batch)
    hist = []
    step = 0
    for ep in range(epochs):
        perm = torch.randperm(n, generator=gen).cuda()
        tot = 0.0
        for b0 in range(0, n - batch + 1, batch):
            idx = perm[b0: b0 + batch]
            x = inputs.index_select(0, idx).contiguous()
            t = tgt.index_select(0, idx).contiguous()
            cur_lr = lr * 0.5 * (1.0 + math.cos(math.pi * step / max(steps, 1)))  # cosine decay
            net.train_step(x, t, cur_lr, loss)
            tot += float(loss.item()) if (b0 // batch) % 50 == 0 else 0.0
            step += 1
        hist.append(tot)
        if log:
            log(f"epoch {ep}: sampled loss {float(loss.item()):.4f}")
    return net.get_params(), hist


def predict(params: np.ndarray, inputs, batch: int = 256) -> np.ndarray:
    """Twists predicted for `inputs` (outputs times the stored scale)."""
    import torch

    from . import initnet as IN

    net = IN.InitNet(max_batch=batch)
    net.set_params(params)
    off, wfc, bfc, sc, total = IN.layout()
    scale = params[sc: sc + 6]
    out = []
    for b0 in range(0, inputs.shape[0], batch):
        x = inputs[b0: b0 + batch].contiguous()
        out.append(net.forward(x).cpu().numpy())
    torch.cuda.synchronize()
    return np.concatenate(out) * scale[None]


def twist_errors(pred: np.ndarray, label: np.ndarray):
    """Rotation (deg) and translation (mm) of exp(pred)^-1 exp(label), per sample."""
    Tp, Tl = se3_exp(pred), se3_exp(label)
    out = np.zeros((len(pred), 2))
    for i in range(len(pred)):
        D = np.linalg.inv(Tp[i]) @ Tl[i]
        c = np.clip((np.trace(D[:3, :3]) - 1) / 2, -1, 1)
        out[i] = [math.degrees(math.acos(c)), np.linalg.norm(D[:3, 3])]
    return out[:, 0], out[:, 1]


def time_steps(steps: int, batch: int = 256, warmup: int = 3) -> dict:
    """Milliseconds per training step (forward, backward, Adam) and per
    forward pass of a batch, on random inputs, timed with CUDA events on the
    network's stream after `warmup` steps."""
    import torch

    from . import initnet as IN

    rng = np.random.default_rng(0)
    net = IN.InitNet(max_batch=batch)
    net.set_params(IN.init_params(1))
    x = torch.from_numpy(rng.uniform(0, 1, size=(batch, 60, 80, 4)).astype(np.float32))
    x = x.to(torch.bfloat16).cuda().contiguous()
    t = torch.from_numpy(rng.normal(size=(batch, 6)).astype(np.float32)).cuda()
    loss = torch.zeros(1, device="cuda")
    for _ in range(warmup):
        net.train_step(x, t, 1e-4, loss)

    def timed(fn):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        for _ in range(steps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / steps

    return {"batch": batch, "train_step_ms": timed(lambda: net.train_step(x, t, 1e-4, loss)),
            "forward_ms": timed(lambda: net.forward(x))}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--time-steps", type=int, default=0, help="only time this many training steps")
    ap.add_argument("--batch", type=int, default=256)
    ap.add_argument("--pairs", type=int, default=200000)
    ap.add_argument("--val", type=int, default=2048)
    ap.add_argument("--epochs", type=int, default=8)
    ap.add_argument("--seed", type=int, default=20000)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--out", default=None)
    a = ap.parse_args()
    if a.time_steps > 0:
        print(time_steps(a.time_steps, a.batch))
        return
    if not a.out:
        ap.error("--out is required to train")
    t0 = time.time()
    x, tw, _ = make_pairs(a.pairs, a.seed)
    xv, twv, _ = make_pairs(a.val, a.seed + 500000)
    t1 = time.time()
    params, hist = train(x, tw, a.epochs, lr=a.lr, seed=a.seed)
    t2 = time.time()
    pv = predict(params, xv)
    er, et = twist_errors(pv, twv)
    zr, zt = twist_errors(np.zeros_like(twv), twv)
    np.savez(a.out, params=params, pairs=a.pairs, epochs=a.epochs, seed=a.seed,
             val_rot_deg_median=np.median(er), val_trans_mm_median=np.median(et))
    print(f"data {t1 - t0:.0f} s, training {t2 - t1:.0f} s; validation ({a.val} pairs): "
          f"predicted rot {np.median(er):.3f} deg / trans {np.median(et):.2f} mm (median), "
          f"identity rot {np.median(zr):.3f} deg / trans {np.median(zt):.2f} mm")


if __name__ == "__main__":
    main()
