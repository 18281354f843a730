"""The tile-shape autotuner: every ICP chunks-per-CTA choice gives the same
poses bit for bit (the normal equations are exact integer sums), and the tuner
leaves its choice set on the batch."""
import numpy as np
import pytest

import recon_gb300 as rg
from scenes import frame_pair, n_select_for
from test_gpu_parity import assert_bitexact

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _batch():
    pairs = [frame_pair(320, 240, seed=61), frame_pair(160, 120, seed=62)]
    cfgs = [rg.make_config(p.W, p.H, p.L, mode=rg.BIOBJECTIVE, iters=(2, 3, 4), n_select=n_select_for(p.W, p.H))
            for p in pairs]
    b = rg.Batch(cfgs, [p.cal.calib for p in pairs])
    b.set_reference([p.g0 for p in pairs], [p.d0 for p in pairs])
    b.set_current([p.g1 for p in pairs], [p.d1 for p in pairs])
    return b


def test_chunks_per_cta_do_not_change_poses():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    b = _batch()
    T0 = np.tile(np.eye(4, dtype=np.float32), (2, 1, 1))
    ref, _ = b.track(T0)
    for c in (1, 2, 5, 64):
        b.set_icp_chunks_per_cta([c, c, c, c])
        assert b.icp_chunks_per_cta()[:3] == [c, c, c]
        T, _ = b.track(T0)
        assert_bitexact(T, ref, f"{c} chunks per CTA")
    with pytest.raises(rg.ReconError):
        b.set_icp_chunks_per_cta([65, 0, 0, 0])


def test_autotune_picks_from_candidates_and_keeps_poses():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from recon_gb300.tune import autotune_icp_chunks
    b = _batch()
    T0 = np.tile(np.eye(4, dtype=np.float32), (2, 1, 1))
    ref, _ = b.track(T0)
    chosen, table = autotune_icp_chunks(b, candidates=(1, 2, 4), reps=1)
    assert sorted(table) == [0, 1, 2]
    for l in range(3):
        assert chosen[l] in (1, 2, 4) and set(table[l]) == {1, 2, 4}
    assert b.icp_chunks_per_cta()[:3] == chosen[:3]
    T, _ = b.track(T0)
    assert_bitexact(T, ref, "poses after tuning")
