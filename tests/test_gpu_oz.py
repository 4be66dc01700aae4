"""The tensor-core GEMM of the mixed form (k_oz_slice + k_oz_gemm: digit-sliced BF16
products accumulated exactly in FP32 on tcgen05, recombined in integer arithmetic),
through the C ABI entry alfgpu_oz_dgemm, against an extended-precision product.

Bound per element (the scheme's truncation of both operands at 2^-54 relative to their
row / column scale, plus the final rounding):
    |C - AB| <= 2^-52 (max_k |A_ik| sum_k |B_kj| + sum_k |A_ik| max_k |B_kj|) + 2^-53 |AB|
"""
import ctypes as C

import numpy as np
import pytest

from alf_gb300 import _lib

pytestmark = pytest.mark.gpu


def _oz(A, B):
    L = _lib.lib()
    A = np.asfortranarray(A, dtype=np.float64)
    B = np.asfortranarray(B, dtype=np.float64)
    m, k = A.shape
    n = B.shape[1]
    Cm = np.zeros((m, n), dtype=np.float64, order="F")
    rc = L.alfgpu_oz_dgemm(m, n, k, A.ctypes.data, m, B.ctypes.data, k, Cm.ctypes.data, m, 0)
    assert rc == 0, rc
    return Cm


def _exact(A, B):
    # np.longdouble carries 64 (x86) or 113 (aarch64) significant bits: 2^-11 or less of the bound
    return A.astype(np.longdouble) @ B.astype(np.longdouble)


@pytest.mark.parametrize("m,n,k", [(7, 5, 9), (130, 70, 200), (256, 256, 256), (300, 200, 288), (64, 96, 448),
                                   (33, 40, 500)])
def test_oz_dgemm_random(m, n, k):
    r = np.random.default_rng(m * 1000 + n + k)
    A = r.standard_normal((m, k)) * np.exp(r.uniform(-8, 0, (m, k)))
    B = r.standard_normal((k, n))
    Cg = _oz(A, B)
    Ce = _exact(A, B)
    aA, aB = np.abs(A), np.abs(B)
    bound = 2.0 ** -52 * (aA.max(1)[:, None] * aB.sum(0)[None, :] + aA.sum(1)[:, None] * aB.max(0)[None, :]) \
        + 2.0 ** -53 * np.abs(Ce).astype(np.float64)
    err = np.abs(Cg.astype(np.longdouble) - Ce).astype(np.float64)
    assert np.all(err <= bound), float((err / bound).max())


def test_oz_dgemm_integers_exact():
    # small integers: every digit product and sum is exact, so is the result
    r = np.random.default_rng(7)
    A = r.integers(-1000, 1000, (150, 256)).astype(np.float64)
    B = r.integers(-1000, 1000, (256, 90)).astype(np.float64)
    assert np.array_equal(_oz(A, B), A @ B)


def test_oz_dgemm_zero_rows_and_scales():
    r = np.random.default_rng(9)
    A = r.standard_normal((100, 64))
    A[5] = 0.0
    A[7] *= 1e-200
    A[9] *= 1e200
    B = r.standard_normal((64, 50))
    B[:, 3] = 0.0
    Cg = _oz(A, B)
    Ce = (A.astype(np.longdouble) @ B.astype(np.longdouble)).astype(np.float64)
    assert np.all(Cg[5] == 0.0) and np.all(Cg[:, 3] == 0.0)
    rel = np.abs(Cg - Ce) / (np.abs(A).max(1)[:, None] * np.abs(B).sum(0)[None, :] + 1e-300)
    assert rel.max() < 2.0 ** -50
