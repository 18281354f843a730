"""Mixed-precision tracking on the GPU (RECON_PRECISION_MIXED: FP16 current
images and reference intensities, BF16 photometric Jacobians, FP32 arithmetic,
exact fixed-point sums, FP64 solve) against the oracle's mixed-precision mode,
which rounds the same arrays the same way: every iteration must be identical.
The pose difference to the FP32 path is the precision's own cost."""
import numpy as np
import pytest

import oracle_lib as O
import recon_gb300 as rg
from scenes import frame_pair, n_select_for
from test_gpu_parity import assert_bitexact, compare_traces

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.mark.parametrize("W,H,mode,iters,bins", [(320, 240, rg.PHOTOMETRIC, (10, 10, 10), 256),
                                                 (320, 240, rg.PHOTOMETRIC, (10, 10, 10), 64),
                                                 (640, 480, rg.BIOBJECTIVE, (1, 3, 10, 5), 64)])
def test_mixed_precision_matches_mixed_oracle(W, H, mode, iters, bins):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    p = frame_pair(W, H, seed=81)
    P = n_select_for(W, H)
    poses = {}
    for prec in (rg.PRECISION_FP32, rg.PRECISION_MIXED):
        cfg = rg.make_config(W, H, p.L, mode=mode, iters=iters, n_select=P, hist_bins=bins, precision=prec)
        trk = rg.Tracker(cfg, p.cal.calib)
        trk.enable_trace(64)
        trk.set_reference(p.g0, p.d0)
        trk.set_current(p.g1, p.d1)
        T, _ = trk.track()
        orc = O.OracleTracker(O.make_config(W, H, p.L, mode=mode, iters=iters, n_select=P, hist_bins=bins,
                                            precision=prec), p.cal.calib)
        orc.set_reference(p.g0, p.d0)
        orc.set_current(p.g1, p.d1)
        To, tro = orc.track()
        compare_traces(trk.trace(0), tro)
        assert_bitexact(T, To, f"final pose (precision {prec})")
        poses[prec] = T.astype(np.float64)
    from recon_gb300 import synth
    mm, deg = synth.pose_error(poses[rg.PRECISION_MIXED], poses[rg.PRECISION_FP32])
    assert mm < 1.0 and deg < 0.05, (mm, deg)


def test_bad_precision_is_rejected():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    cfg = rg.make_config(320, 240, 3, precision=2)
    with pytest.raises(rg.ReconError):
        rg.Tracker(cfg, frame_pair(320, 240, seed=1).cal.calib)
