"""The host eigensystem behind the transition matrices (Householder reduction
and symmetric QR, messi_host_reversible_eig): no GPU.  Reconstruction,
orthonormality and the eigenvalues against numpy's symmetric solver, for
GTR (4 states) and muse (16 states, the rate matrices of the pair model,
restated in the oracle from src/RateMatrices.jl:69-148) matrices, including
repeated eigenvalues; invalid inputs are rejected."""
import ctypes

import numpy as np
import pytest

from messi_gb300 import _lib
from oracle import c_oracle as co


def _eig(Q, pi):
    lib = _lib.load()
    n = len(pi)
    Q = np.ascontiguousarray(Q, np.float64)
    pi = np.ascontiguousarray(pi, np.float64)
    w = np.zeros(n)
    U = np.zeros(n * n)
    rc = lib.messi_host_reversible_eig(n, Q.ctypes.data, pi.ctypes.data, w.ctypes.data, U.ctypes.data)
    return rc, w, U.reshape(n, n)


def _check(Q, pi):
    rc, w, U = _eig(Q, pi)
    assert rc == 0
    n = len(pi)
    d = np.sqrt(pi)
    A = d[:, None] * Q / d[None, :]
    A = 0.5 * (A + A.T)
    scale = max(1.0, np.abs(A).max())
    np.testing.assert_allclose(U.T @ U, np.eye(n), atol=1e-13)
    np.testing.assert_allclose(U @ np.diag(w) @ U.T, A, atol=1e-12 * scale)
    np.testing.assert_allclose(np.sort(w), np.linalg.eigvalsh(A), atol=1e-12 * scale)
    # P = D^-1/2 U exp(W t) U^T D^1/2 is a stochastic matrix
    P = (1 / d)[:, None] * (U @ np.diag(np.exp(w * 0.3)) @ U.T) * d[None, :]
    np.testing.assert_allclose(P.sum(axis=1), 1.0, atol=1e-12)


@pytest.mark.parametrize("seed", range(6))
def test_gtr_matrices(seed):
    rng = np.random.default_rng(seed)
    q = rng.uniform(0.2, 3.0, 6)
    pi = rng.dirichlet([4.0] * 4)
    _check(co.gtr(q, pi), pi)


@pytest.mark.parametrize("seed", range(6))
def test_muse_matrices(seed):
    rng = np.random.default_rng(100 + seed)
    q = rng.uniform(0.2, 3.0, 6)
    pi4 = rng.dirichlet([4.0] * 4)
    lam = rng.uniform(1.0, 5.0, 3)
    sr1, sr2 = rng.uniform(0.1, 3.0, 2)
    Q = co.muse(lam[0], lam[1], lam[2], q, pi4, sr1, sr2)
    pi16 = co.musefreqs(pi4, lam[0], lam[1], lam[2])
    _check(Q, pi16)


def test_lambda_one_and_equal_rates_repeat_eigenvalues():
    # lambda = 1 and equal site rates: the pair process is two independent
    # copies of one GTR process, so eigenvalues repeat
    q = np.ones(6)
    pi4 = np.full(4, 0.25)
    Q = co.muse(1.0, 1.0, 1.0, q, pi4, 1.0, 1.0)
    pi16 = co.musefreqs(pi4, 1.0, 1.0, 1.0)
    _check(Q, pi16)
    rc, w, _ = _eig(Q, pi16)
    assert len(np.unique(np.round(w, 9))) < 16


def test_invalid_inputs_are_rejected():
    Q = co.gtr(np.ones(6), np.full(4, 0.25))
    assert _eig(Q, np.array([0.5, 0.5, 0.0, 0.0]))[0] == _lib.MESSI_EINVAL
    bad = Q.copy()
    bad[0, 1] = np.nan
    assert _eig(bad, np.full(4, 0.25))[0] == _lib.MESSI_EINVAL
    lib = _lib.load()
    z = np.zeros(17 * 17)
    assert lib.messi_host_reversible_eig(17, z.ctypes.data, z.ctypes.data, z.ctypes.data, z.ctypes.data) == \
        _lib.MESSI_EINVAL
