"""The truncation of the Student-t variance sums
(recon_gb300/csrc/exact_arith.cuh) against the conversion it replaces.

On the host: the method restated in C (exact_arith_check.c) over a dense sweep
of [0, 2^23).  On the GPU: the device code itself over every float of
[0, 2^23) (recon_selftest_exact_arith).  The end-to-end effect (ICP weights and
variance sums identical to the oracle's) is covered by the parity tests.
"""
import os
import shutil
import subprocess

import pytest

import recon_gb300 as rg

HERE = os.path.dirname(os.path.abspath(__file__))


def test_exact_arith_method_on_host():
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    out = os.path.join(HERE, "_build")
    os.makedirs(out, exist_ok=True)
    exe = os.path.join(out, "exact_arith_check")
    subprocess.run([cc, "-O2", "-ffp-contract=off", os.path.join(HERE, "exact_arith_check.c"), "-o", exe, "-lm"],
                   check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith("trunc 0/")


def test_selftest_symbol_is_exported():
    assert hasattr(rg.lib(), "recon_selftest_exact_arith")


@pytest.mark.gpu
def test_exact_arith_on_gpu():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    assert rg.selftest_exact_arith() == 0
