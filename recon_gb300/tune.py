"""Autotuner for the tile shape of the linearisation kernel.

k_iter gives each CTA a number of 1024-pixel ICP chunks per pyramid level.
Fewer chunks per CTA means more CTAs (more parallelism, more per-CTA fixed
cost: descriptor load, shared sums, integer atomics); more chunks amortise that
cost over a longer serial loop.  The normal equations are exact integer sums,
so every choice gives bit-identical poses and only the speed differs, which
makes a timing search safe to run on live data.

The search is coordinate-wise, coarse level to fine: for each level it times
whole tracking runs of the batch's current frame pair with each candidate (the
other levels fixed at their best so far) and keeps the fastest.  Each run
starts from the same initial pose, so each one does the same work.
"""
from __future__ import annotations

import numpy as np


def autotune_icp_chunks(batch, candidates=(1, 2, 3, 4, 6, 8), reps: int = 3, T_init=None):
    """Picks the ICP chunks per CTA of every level of `batch` by timing and
    leaves them set.  The batch must hold a reference and a current frame.
    Returns (chosen per-level values, {level: {candidate: ms}})."""
    if T_init is None:
        T_init = np.tile(np.eye(4, dtype=np.float32), (batch.n, 1, 1))
    chosen = batch.icp_chunks_per_cta()
    levels = [l for l in range(4) if chosen[l] > 0]
    table = {}
    batch.enable_timing(True)
    try:
        batch.track(T_init)  # warm-up
        for level in sorted(levels, reverse=True):
            table[level] = {}
            for c in candidates:
                trial = list(chosen)
                trial[level] = c
                batch.set_icp_chunks_per_cta(trial)
                batch.timing(reset=True)
                for _ in range(reps):
                    batch.track(T_init)
                ms, _ = batch.timing(reset=True)["gn_iteration"]
                table[level][c] = ms / reps
            chosen[level] = min(table[level], key=table[level].get)
    finally:
        batch.set_icp_chunks_per_cta(chosen)
        batch.enable_timing(False)
    return chosen, table
