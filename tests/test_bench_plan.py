"""Host logic of the benchmark step: the frame plan of one step (every
segment's keyframe, then frame s of every segment per sequence position), the
keyframe fusion between the two halves of each segment, and the scatter of the
tracked poses back to frame order.  A recording stand-in for the batch checks
the indices handed to the frame-stack calls; no GPU."""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


class RecordingBatch:
    def __init__(self):
        self.calls = []

    def set_reference_frames(self, g, d, index):
        self.calls.append(("ref", np.asarray(index).copy()))

    def track_sequence_frames(self, g, d, index):
        idx = np.asarray(index)
        self.calls.append(("seq", idx.copy()))
        # pose of frame f: a matrix filled with f, so the scatter is visible
        T = np.broadcast_to(idx[:, :, None, None].astype(np.float32), idx.shape + (4, 4)).copy()
        self.last_frames = idx.shape[0]
        return T, []

    def fuse_sequence(self, nframes, gate_mm):
        assert nframes <= self.last_frames
        self.calls.append(("fuse", nframes, gate_mm))


def test_plan_of_the_benchmark_trajectory():
    segs = bench.segments(300)
    assert len(segs) == 30 and all(len(fr) == 10 for _, fr in segs)
    ref, seq, own = bench.step_plan(segs)
    assert ref.tolist() == list(range(0, 300, 10))
    assert seq.shape == (10, 30) and own.all()
    assert seq[0].tolist() == [k + 1 for k in range(0, 300, 10)]
    assert sorted(seq.reshape(-1).tolist()) == [f for k in range(0, 300, 10) for f in range(k + 1, k + 11)]


def test_short_last_segment_repeats_its_last_frame():
    segs = bench.segments(25)  # keyframes 0, 10, 20; the last segment tracks 21..25
    ref, seq, own = bench.step_plan(segs)
    assert ref.tolist() == [0, 10, 20]
    assert seq.shape == (10, 3)
    assert seq[:, 2].tolist() == [21, 22, 23, 24, 25, 25, 25, 25, 25, 25]
    assert own[:, 2].tolist() == [True] * 5 + [False] * 5
    assert own[:, :2].all()


def test_run_step_scatters_every_tracked_frame_once():
    segs = bench.segments(25)
    plan = bench.step_plan(segs)
    b = RecordingBatch()
    out = np.full((26, 4, 4), -1.0, np.float32)
    bench.run_step(b, plan, None, None, out)
    assert [c[0] for c in b.calls] == ["ref", "seq", "fuse", "seq"]
    assert b.calls[0][1].tolist() == [0, 10, 20]
    # the first five frames of every segment, their fusion, then the rest
    assert np.array_equal(b.calls[1][1], plan[1][:bench.FUSE_FRAMES])
    assert b.calls[2] == ("fuse", bench.FUSE_FRAMES, bench.GATE_MM)
    assert np.array_equal(b.calls[3][1], plan[1][bench.FUSE_FRAMES:])
    tracked = [f for _, fr in segs for f in fr]
    for f in range(26):
        if f in tracked:
            assert (out[f] == f).all(), f
        else:
            assert (out[f] == -1.0).all(), f  # keyframes keep their entry
