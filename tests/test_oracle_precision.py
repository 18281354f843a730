"""The oracle's mixed-precision storage: its FP16 and BF16 rounding (to nearest,
ties to even) against independent implementations (numpy's float16 and
torch's bfloat16 casts) over random bit patterns and the binary16 boundaries
(subnormals, the normal threshold, overflow); and the mixed-precision oracle
tracker against the FP32 one on a frame pair."""
import numpy as np
import pytest

import oracle_lib as O
from scenes import frame_pair, n_select_for


def _samples():
    rng = np.random.default_rng(3)
    bits = np.concatenate([
        rng.integers(0, 2 ** 32, size=60000, dtype=np.uint64).astype(np.uint32),
        np.arange(0x33000000, 0x33000000 + 8192, dtype=np.uint32),   # around 2^-25 (half of the smallest subnormal)
        np.arange(0x387fe000, 0x38802000, dtype=np.uint32),          # the normal threshold 2^-14
        np.arange(0x477fe000, 0x47802000, dtype=np.uint32),          # 65504 .. 65536 (overflow)
        np.arange(0x3f7ff000, 0x3f801000, dtype=np.uint32),          # around 1.0 (images, intensities)
    ])
    x = bits.view(np.float32)
    return x[np.isfinite(x)]


def test_f16_rounding_matches_numpy():
    L = O.lib()
    x = _samples()
    with np.errstate(over="ignore"):
        want = x.astype(np.float16).astype(np.float32)
    got = np.array([L.orc_f16_round(float(v)) for v in x], np.float32)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def test_bf16_rounding_matches_torch():
    torch = pytest.importorskip("torch")
    L = O.lib()
    x = _samples()
    want = torch.from_numpy(x.copy()).to(torch.bfloat16).to(torch.float32).numpy()
    got = np.array([L.orc_bf16_round(float(v)) for v in x], np.float32)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def test_mixed_precision_tracker_stays_close_to_fp32():
    p = frame_pair(320, 240, seed=5)
    out = []
    for prec in (0, 1):
        cfg = O.make_config(320, 240, 3, mode=O.PHOTOMETRIC, iters=(10, 10, 10), n_select=n_select_for(320, 240),
                            precision=prec)
        orc = O.OracleTracker(cfg, p.cal.calib)
        orc.set_reference(p.g0, p.d0)
        orc.set_current(p.g1, p.d1)
        T, _ = orc.track()
        out.append(T.astype(np.float64))
        orc.close()
    from recon_gb300 import synth
    mm, deg = synth.pose_error(out[1], out[0])
    assert not np.array_equal(out[0], out[1])  # the rounding is applied
    assert mm < 1.0 and deg < 0.05, (mm, deg)
