"""What the trained network gains over the tracker without it, on held-out
data.

Two seeded 100-frame trajectories through scenes the network never saw
(training used scene seeds from 20000 up, the benchmark 1000) are tracked by
the benchmark's own step -- keyframe every 10 frames, depth/colour fusion of
the first five frames, bi-objective 640x480 -- on the same shortened schedule
twice: with the learned start pose (recon_gb300/weights/initnet_200k.npz) and
with the previous frame's pose as the start, the reference tracker's rule.
Both are scored against the FP64 oracle run of the same trajectories on the
full schedule.  The network's start must leave more frames within 1 mm /
0.05 deg of the oracle and a lower median error.
"""
import os
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402

HELD_OUT_SEEDS = (4001, 4041)
FRAMES = 100


def track_arms(schedule, seeds=HELD_OUT_SEEDS, frames=FRAMES):
    """Pose errors against the FP64 oracle of the with-network and
    previous-pose arms on `schedule`, over the given trajectories."""
    import recon_gb300 as rg
    import recon_gb300.initnet as IN
    params, _ = bench.load_net_params()
    assert params is not None, "trained weights missing"
    err = {"net": [], "prev": []}
    for seed in seeds:
        cal, scene, poses = bench.make_workload(seed, frames)
        segs = bench.segments(frames)
        plan = bench.step_plan(segs)
        fr = [f for _, x in segs for f in x]
        gray, depth = bench.render_frames_gpu(cal, scene, poses, seed, torch)
        ref64, _ = bench.fp64_trajectory(cal, gray.cpu().numpy(), depth.cpu().numpy().view(np.uint16), segs)
        stream = torch.cuda.Stream()
        batch = bench.make_batch(cal, len(segs), stream.cuda_stream)
        net = IN.InitNet(max_batch=len(segs), stream=stream.cuda_stream)
        net.set_params(params)
        for arm in ("net", "prev"):
            if arm == "net":
                batch.set_init_net(net, schedule)
            else:
                batch.set_init_net(None)
                for i in range(batch.n):
                    batch.set_iterations(i, schedule)
            out = np.zeros((frames + 1, 4, 4), np.float32)
            bench.run_step(batch, plan, gray, depth, out)
            err[arm].append(bench.pose_errors(out, ref64, fr))
        batch.set_init_net(None)
        batch.close()
        net.close()
    return {k: bench.error_summary(np.concatenate(v))[0] for k, v in err.items()}


@pytest.fixture(scope="module", autouse=True)
def cuda_lib():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def test_network_start_beats_previous_pose_start_on_held_out_trajectories():
    res = track_arms(bench.LEARNED_ITERS)
    print("learned start", res["net"], "\nprevious-pose start", res["prev"])
    assert res["net"]["within_bound"] > res["prev"]["within_bound"], res
    assert res["net"]["median_mm"] < res["prev"]["median_mm"], res
