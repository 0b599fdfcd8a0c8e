"""Structures on the GPU: posterior decoding (bit-exact against the FP32
oracle restatement and, where built, the reference's own kernel), the
device-resident consensus chain, and stochastic structure sampling
(empirical pair frequencies against the exact posteriors)."""
import numpy as np
import pytest

from oracle import c_oracle as co
from oracle import ref_kernels as rk

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def api():
    from messi_gb300 import api as _api
    return _api


def _scores(L, W, seed):
    rng = np.random.default_rng(seed)
    u = rng.uniform(-30.0, -8.0, L)
    p = np.full((L, L), -np.inf)
    for i in range(L):
        for j in range(i + 1, min(L, i + W + 1)):
            odds = rng.normal(-2.0, 3.0) + (rng.random() < 0.08) * rng.uniform(6, 18)
            p[i, j] = p[j, i] = u[i] + u[j] + odds
    return u, p


def _posteriors(u, p):
    ins = co.inside(u, p)
    outs = co.outside(ins, u, p)
    return co.basepairprobs(ins, outs, u, p)


@pytest.mark.parametrize("L,W", [(2, 1), (7, 6), (60, 59), (150, 40)])
def test_posterior_decoding_is_bit_exact(api, L, W):
    u, p = _scores(L, W, seed=L + W)
    single, pair = _posteriors(u, p)
    e, s = api.computeposteriordecodingcuda(single, pair, 2.0)
    e_ref, s_ref = co.posterior_decoding(single, pair, 2.0)  # row-major [i, j]
    np.testing.assert_array_equal(e, e_ref.astype(np.float64))
    np.testing.assert_array_equal(s, s_ref)
    paired = api.getPosteriorDecodingConsensusStructure(pair, single)
    np.testing.assert_array_equal(paired, co.posterior_traceback(s_ref))
    # the whole chain on the device gives the same structure
    np.testing.assert_array_equal(api.consensusstructure(u, p), paired)


@pytest.mark.skipif(not rk.available(), reason="reference cubins not built (make -C oracle ref)")
@pytest.mark.parametrize("L", [9, 120])
def test_posterior_decoding_equals_reference_kernel(api, L):
    u, p = _scores(L, L - 1, seed=3 * L)
    single, pair = _posteriors(u, p)
    e_ref, s_ref = rk.posterior_decoding(single, pair, 2.0)
    e, s = api.computeposteriordecodingcuda(single, pair, 2.0)
    np.testing.assert_array_equal(e, e_ref.astype(np.float64))
    np.testing.assert_array_equal(s, s_ref)
    e_o, s_o = co.posterior_decoding(single, pair, 2.0)
    np.testing.assert_array_equal(e_o, e_ref)
    np.testing.assert_array_equal(s_o, s_ref)


@pytest.mark.parametrize("env", [{"MESSI_WAVE_CTAS": "7"}, {"MESSI_WAVE_CTAS": "1"}, {"MESSI_WAVE_THREADS": "1024"}])
def test_posterior_decoding_same_bits_on_any_grid(api, env, monkeypatch):
    """The decoding wavefront takes two diagonals per grid barrier, each CTA
    owning a run of rows (and one more on the pair's first diagonal): with 7
    CTAs or one (rows beyond two per lane group computed whole) or 1,024-
    thread CTAs, e and s equal the oracle's to the bit."""
    L, W = 150, 149
    u, p = _scores(L, W, seed=11)
    single, pair = _posteriors(u, p)
    e_ref, s_ref = co.posterior_decoding(single, pair, 2.0)
    for k, v in env.items():
        monkeypatch.setenv(k, v)
    ctx = api.Context(0)
    try:
        e, s = api.computeposteriordecodingcuda(single, pair, 2.0, ctx=ctx)
    finally:
        ctx.close()
    np.testing.assert_array_equal(e, e_ref.astype(np.float64))
    np.testing.assert_array_equal(s, s_ref)


def _check_structure(row, W):
    L = len(row)
    stack = []
    for c in range(L):
        k = row[c] - 1
        if k < 0:
            continue
        assert row[k] - 1 == c
        if k > c:
            assert 3 <= k - c <= W
            stack.append(k)
        else:
            assert stack and stack[-1] == c  # nested
            stack.pop()
    assert not stack


@pytest.mark.parametrize("L,W", [(24, 23), (40, 12)])
def test_sampled_structures_follow_the_posterior(api, L, W):
    u, p = _scores(L, W, seed=100 + L)
    single, pair = _posteriors(u, p)
    n = 40000
    S, priors = api.samplestructures(u, p, n, seed=7)
    assert S.shape == (n, L) and np.all(np.isfinite(priors))
    for row in S[:500]:
        _check_structure(row, W)
    freq = np.zeros((L, L))
    rows, cols = np.nonzero(S)
    np.add.at(freq, (cols, S[rows, cols] - 1), 1.0)
    freq /= n
    tol = 5.0 * np.sqrt(pair * (1.0 - pair) / n) + 2e-3
    assert np.all(np.abs(freq - pair) <= tol), float(np.max(np.abs(freq - pair) - tol))
    np.testing.assert_allclose(1.0 - freq.sum(axis=1), single, atol=5.0 * np.sqrt(0.25 / n) + 2e-3)
    # the device's prior of each structure equals the host parse (calculateKH99prior)
    from messi_gb300.structures import calculateKH99prior
    for row, pr in zip(S[:200], priors[:200]):
        assert abs(pr - calculateKH99prior(row)) <= 1e-9 * abs(pr)
    # the same seed gives the same structures
    S2, _ = api.samplestructures(u, p, 64, seed=7)
    np.testing.assert_array_equal(S2, S[:64])
