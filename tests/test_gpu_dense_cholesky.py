"""The dense solver's blocked Cholesky on its own (sfmba_dense_cholesky, the
factorisation of crates/sfm-ba/src/lib.rs:1081-1094), with the trailing
updates in FP64 fused multiply-adds and on the BF16 tensor cores by
error-free splitting.

Bars: both factors reproduce A to FP64 backward error (||A - L L^T||_F /
||A||_F below 1e-14, the FP64 factor's own level within a factor of 8);
the two factors agree with each other and with LAPACK's to the forward
error the condition number allows; a matrix that is not positive definite
is reported, not factored."""
import numpy as np
import pytest

from sfmtory_gb300 import native

pytestmark = pytest.mark.gpu


def _spd(n, seed, row_scale_decades=0.0):
    rng = np.random.default_rng(seed)
    M = rng.standard_normal((n, n + 8))
    A = M @ M.T / n + 1e-3 * np.eye(n)
    if row_scale_decades:
        d = 10.0 ** rng.uniform(-row_scale_decades, row_scale_decades, n)
        A = d[:, None] * A * d[None, :]
    return A


def _backward(A, L):
    return np.linalg.norm(A - L @ L.T) / np.linalg.norm(A)


@pytest.mark.parametrize("n,decades", [(64, 0.0), (130, 0.0), (1000, 0.0), (2000, 0.0), (1037, 3.0)])
def test_tensor_update_reproduces_fp64_factor(n, decades):
    A = _spd(n, seed=n, row_scale_decades=decades)
    Lf, _ = native.dense_cholesky(A, tensor_update=False)
    Lt, _ = native.dense_cholesky(A, tensor_update=True)
    bf, bt = _backward(A, Lf), _backward(A, Lt)
    assert bf < 1e-14 and bt < 1e-14, (bf, bt)
    assert bt <= 8 * bf + 1e-16, (bf, bt)
    Ln = np.linalg.cholesky(A)
    scale = np.abs(Ln).max()
    cond_bound = 1e-16 * np.linalg.cond(A) * 10
    assert np.abs(Lf - Ln).max() / scale < max(cond_bound, 1e-13)
    assert np.abs(Lt - Ln).max() / scale < max(cond_bound, 1e-13)
    assert np.all(np.triu(Lt, 1) == 0.0)


def test_not_positive_definite_is_reported():
    A = _spd(200, seed=3)
    A[150, 150] = -1.0
    for tensor in (False, True):
        with pytest.raises(native.SfmbaError, match="positive definite"):
            native.dense_cholesky(A, tensor_update=tensor)


def test_peaks_are_positive():
    pk = native.measure_peaks()
    assert pk["dfma_tflops"] > 0.1 and pk["dmma_tflops"] > 0.1 and pk["bf16_mma_tflops"] > 10.0, pk
