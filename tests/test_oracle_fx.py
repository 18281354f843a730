"""The oracle's exact fixed-point reduction and its FP64 solve / exponential.

The tracker's 27 normal-equation terms are the exact sum of the FP32 warp
values of the canonical order, rounded once to FP64.  These tests check that
definition against Python's math.fsum (an exactly rounded float sum), its
independence of the order of addition, its range limits, and the LDL^T solve
and Pade exponential against numpy / scipy.
"""
import ctypes
import math

import numpy as np
import pytest

import oracle_lib as O
from oracle_lib import ptr as p

FX_BYTES = 27 * 4 * 8 + 8


def fx_sum(values):
    L = np.zeros(4, np.int64)
    bad = np.zeros(1, np.int32)
    lib = O.lib()
    for v in values:
        lib.orc_fx_add(p(L), ctypes.c_float(float(v)), p(bad))
    return lib.orc_fx_to_double(p(L)), int(bad[0])


def test_fx_sum_is_exactly_rounded():
    rng = np.random.default_rng(11)
    for trial in range(40):
        n = int(rng.integers(1, 400))
        exps = rng.integers(-40, 46, size=n)
        v = (rng.uniform(-1, 1, size=n) * np.exp2(exps)).astype(np.float32)
        got, bad = fx_sum(v)
        assert bad == 0
        want = math.fsum(float(x) for x in v)
        assert got == want, (trial, got, want)


def test_fx_sum_with_cancellation():
    v = np.array([3.0e10, 1.0, -3.0e10, 2.0 ** -30, -1.0], np.float32)
    got, _ = fx_sum(v)
    assert got == math.fsum(float(x) for x in v) == 2.0 ** -30


def test_fx_sum_independent_of_order():
    rng = np.random.default_rng(12)
    v = (rng.normal(size=3000) * np.exp2(rng.integers(-60, 40, size=3000))).astype(np.float32)
    a, _ = fx_sum(v)
    b, _ = fx_sum(v[::-1])
    c, _ = fx_sum(rng.permutation(v))
    assert np.float64(a).view(np.uint64) == np.float64(b).view(np.uint64) == np.float64(c).view(np.uint64)


def test_fx_truncates_below_2_pow_minus_64():
    got, bad = fx_sum(np.array([2.0 ** -70, -(2.0 ** -66)], np.float32))
    assert bad == 0 and got == 0.0
    got, _ = fx_sum(np.array([np.float32(1.75 * 2.0 ** -63)], np.float32))
    assert got == 1.5 * 2.0 ** -63  # bits below 2^-64 dropped toward zero
    got, _ = fx_sum(np.array([-np.float32(1.75 * 2.0 ** -63)], np.float32))
    assert got == -1.5 * 2.0 ** -63


@pytest.mark.parametrize("v", [np.inf, -np.inf, np.nan, 2.0 ** 48, -(2.0 ** 50)])
def test_fx_flags_out_of_range(v):
    _, bad = fx_sum(np.array([1.0, v], np.float32))
    assert bad == 1


def test_fx_largest_in_range_value():
    big = np.nextafter(np.float32(2.0 ** 48), np.float32(0))
    got, bad = fx_sum(np.array([big] * 1000, np.float32))
    assert bad == 0 and got == 1000.0 * float(big)


def test_reduce27_fx_matches_fp64_fold():
    rng = np.random.default_rng(13)
    N = 8192
    J = [rng.normal(size=N).astype(np.float32) for _ in range(6)]
    r = rng.normal(size=N).astype(np.float32)
    acc = np.zeros(FX_BYTES, np.uint8)
    A = np.zeros(36)
    b = np.zeros(6)
    A2 = np.zeros(36)
    b2 = np.zeros(6)
    lib = O.lib()
    Jp = O.ptrs(J)
    lib.orc_fx27_clear(p(acc))
    lib.orc_reduce27_fx(Jp, p(r), N, p(acc))
    lib.orc_fx27_value(p(acc), p(A), p(b))
    lib.orc_reduce27(Jp, p(r), N, p(A2), p(b2))
    np.testing.assert_allclose(A, A2, rtol=1e-12, atol=1e-9)
    np.testing.assert_allclose(b, b2, rtol=1e-12, atol=1e-9)
    assert np.array_equal(A.reshape(6, 6), A.reshape(6, 6).T)


def test_cholesky_ldlt_solves():
    rng = np.random.default_rng(14)
    lib = O.lib()
    for _ in range(50):
        M = rng.normal(size=(6, 6))
        A = (M @ M.T + 6 * np.eye(6)) * 10.0 ** rng.uniform(-3, 3)
        b = rng.normal(size=6)
        x = np.zeros(6)
        A64 = np.ascontiguousarray(A)
        assert lib.orc_solve_cholesky(p(A64), p(b), p(x)) == 0
        np.testing.assert_allclose(A @ x, b, rtol=1e-10, atol=1e-10 * np.abs(b).max())
    A = -np.eye(6)
    x = np.ones(6)
    assert lib.orc_solve_cholesky(p(A), p(b), p(x)) == -1
    assert np.all(x == 0)


def test_expm_twist_matches_scipy():
    scipy_linalg = pytest.importorskip("scipy.linalg")
    rng = np.random.default_rng(15)
    lib = O.lib()
    for k in range(40):
        w = rng.normal(size=3) * (10.0 ** rng.uniform(-4, 0.5))
        t = rng.normal(size=3) * (10.0 ** rng.uniform(-4, 0.5))
        A = np.array([[0, -w[2], w[1], t[0]], [w[2], 0, -w[0], t[1]], [-w[1], w[0], 0, t[2]], [0, 0, 0, 0]])
        E = np.zeros(16)
        A64 = np.ascontiguousarray(A.reshape(-1))
        lib.orc_expm_twist(p(A64), p(E))
        np.testing.assert_allclose(E.reshape(4, 4), scipy_linalg.expm(A), rtol=0, atol=1e-13 * max(1, np.abs(A).max() ** 2))
