"""GPU parity against the FP64 oracle, through the C ABI.

Tolerances (spec: the FP32 GPU path within 1e-6 relative
log-likelihood of the FP64 reference):
  * pair log-likelihoods, unpaired log-likelihoods, Z: relative 1e-6
  * inside/outside table cells in the band: |d| <= 1e-6 |ref| + 2e-3
  * posteriors: absolute 1e-4.  Inside/outside cells are FP32 log-odds
    against the unpaired baseline; their magnitude grows with the pairing
    log-odds inside a span (a few hundred nats in these cases), so a stored
    cell carries ~|x| * 2^-24 absolute error and a posterior built from three
    of them ~1e-5 relative.
"""
import numpy as np
import pytest

from oracle import c_oracle as co
from oracle import model_ref as mr

pytestmark = pytest.mark.gpu

REL = 1e-6
POST_TOL = 1e-4


@pytest.fixture(scope="module")
def api():
    from messi_gb300 import api as _api
    return _api


def _params(s):
    from messi_gb300 import model as M
    return M.getparams(s.params15, s.dataset.branchlengths)


def _oracle_pairs(s, W, pairmask=None, per_lambda=False):
    ds = s.dataset
    rp = mr.getparams(s.params15, ds.branchlengths)
    return mr.pair_loglik(ds.tree_arrays(), ds.masks, rp, W, pairmask=pairmask, per_lambda=per_lambda)


def _assert_loglik_close(got, ref, rel=REL):
    fin = np.isfinite(ref)
    assert np.array_equal(fin, np.isfinite(got)), "finite pattern differs"
    assert np.all(np.isneginf(got[~fin]))
    err = np.abs(got[fin] - ref[fin]) / np.maximum(np.abs(ref[fin]), 1.0)
    assert err.max() <= rel, f"max relative error {err.max():.3e}"


def test_unpaired_matches_oracle(api, c1, tiny):
    for s in (tiny, c1):
        ds = s.dataset
        u = api.computeunpairedlikelihoods(ds, _params(s))
        ref, _ = mr.unpaired_loglik(ds.tree_arrays(), ds.masks, mr.getparams(s.params15, ds.branchlengths))
        np.testing.assert_allclose(u, ref, rtol=1e-11)


def test_pairs_match_oracle_all_pairs(api, c1):
    mat, _ = api.felsensteincuda(c1.dataset, _params(c1), None, c1.W)
    ref, _ = _oracle_pairs(c1, c1.W)
    _assert_loglik_close(mat, ref)
    assert np.array_equal(mat, mat.T)


def test_pairs_banded_masked_and_per_lambda(api, c1):
    L = c1.dataset.numcols
    rng = np.random.default_rng(4)
    mask = (rng.random((L, L)) < 0.8).astype(np.uint8)
    mask = np.triu(mask, 1)
    mask = mask + mask.T
    mat, per = api.felsensteincuda(c1.dataset, _params(c1), None, 17, True, pairmask=mask)
    ref, refl = _oracle_pairs(c1, 17, pairmask=mask, per_lambda=True)
    _assert_loglik_close(mat, ref)
    assert len(per) == 5
    for k in range(5):
        _assert_loglik_close(per[k], refl[k])


def test_pairs_tiny_tree(api, tiny):
    mat, _ = api.felsensteincuda(tiny.dataset, _params(tiny), None, tiny.W)
    ref, _ = _oracle_pairs(tiny, tiny.W)
    _assert_loglik_close(mat, ref)


def _random_scores(L, W, seed, strong=0.05):
    """Unpaired / pair log-likelihoods with the magnitudes of a 64-sequence
    alignment: pair scores near u_i + u_j with a few strongly coevolving pairs."""
    rng = np.random.default_rng(seed)
    u = rng.uniform(-80.0, -20.0, L)
    p = np.full((L, L), -np.inf)
    for i in range(L):
        for j in range(i + 1, min(L, i + W + 1)):
            odds = rng.normal(-3.0, 4.0) + (rng.random() < strong) * rng.uniform(10, 40)
            p[i, j] = p[j, i] = u[i] + u[j] + odds
    return u, p


SCFG_CASES = [(1, 1), (2, 1), (3, 2), (5, 4), (17, 5), (40, 39), (64, 10), (97, 3), (130, 40), (200, 199)]


@pytest.mark.parametrize("L,W", SCFG_CASES)
def test_inside_Z_matches_oracle(api, L, W):
    u, p = _random_scores(L, W, seed=L * 1000 + W)
    Z = api.computeinsideKH99(u, p)
    Zref = co.inside(u, p)[0, 0, L - 1]
    assert abs(Z - Zref) <= REL * abs(Zref), (Z, Zref)
    # an explicit band at least as wide as the data gives the same Z
    Z2 = api.computeinsideKH99(u, p, maxspan=min(L - 1, W + 3))
    assert abs(Z2 - Zref) <= REL * abs(Zref)


def _table_close(got, ref, band):
    L = ref.shape[1]
    i, j = np.meshgrid(np.arange(L), np.arange(L), indexing="ij")
    sel = (j >= i) & (j - i <= band)
    for X in range(3):
        g, r = got[X][sel], ref[X][sel]
        fin = np.isfinite(r)
        assert np.array_equal(fin, np.isfinite(g)), f"finite pattern differs for nonterminal {X}"
        d = np.abs(g[fin] - r[fin])
        assert np.all(d <= 1e-6 * np.abs(r[fin]) + 2e-3), f"nonterminal {X}: max abs err {d.max():.3e}"
    # the suffix column (S on the last column) is kept at every span
    fin = np.isfinite(ref[0][:, L - 1])
    d = np.abs(got[0][fin, L - 1] - ref[0][fin, L - 1])
    assert np.all(d <= 1e-6 * np.abs(ref[0][fin, L - 1]) + 2e-3)


@pytest.mark.parametrize("L,W", [(17, 5), (64, 10), (130, 40), (60, 59)])
def test_inside_and_outside_tables(api, L, W):
    u, p = _random_scores(L, W, seed=7 * L + W)
    ins = api.computeinsideKH99(u, p, 1.0, False)
    ref_in = co.inside(u, p)
    _table_close(ins, ref_in, W)
    outs = api.computeoutsideKH99(ref_in, u, p)
    ref_out = co.outside(ref_in, u, p)
    _table_close(outs, ref_out, W)


@pytest.mark.parametrize("L,W", [(9, 8), (40, 12), (130, 40), (100, 99)])
def test_posteriors_match_oracle(api, L, W):
    u, p = _random_scores(L, W, seed=11 * L + W)
    ins = co.inside(u, p)
    outs = co.outside(ins, u, p)
    s_ref, p_ref = co.basepairprobs(ins, outs, u, p)
    s1, p1 = api.computebasepairprobs(ins, outs, u, p)
    assert np.abs(s1 - s_ref).max() < POST_TOL and np.abs(p1 - p_ref).max() < POST_TOL
    Z, s2, p2 = api.computeposteriors(u, p)
    assert abs(Z - ins[0, 0, L - 1]) <= REL * abs(ins[0, 0, L - 1])
    assert np.abs(s2 - s_ref).max() < POST_TOL and np.abs(p2 - p_ref).max() < POST_TOL
    np.testing.assert_allclose(s2 + p2.sum(axis=1), 1.0, atol=1e-5)


def test_structure_integrated_likelihood_matches_oracle(api, c1):
    ds = c1.dataset
    params = _params(c1)
    ll = api.computestructureintegratedlikelihood(ds, params, c1.W)
    ref, info = mr.structure_integrated_likelihood(ds.tree_arrays(), ds.masks, ds.gapfrequency, c1.params15, c1.W)
    assert abs(ll - ref) <= REL * abs(ref), (ll, ref)
    # same through the drop-in call sequence of src/MESSI.jl:305-311
    u = api.computeunpairedlikelihoods(ds, params)
    pmat, _ = api.felsensteincuda(ds, params, None, c1.W)
    api.maskgapped(pmat, ds.gapfrequency, 1.0, -np.inf)
    Z = api.computeinsideKH99(u, pmat)
    assert abs(Z - info["Z"]) <= REL * abs(info["Z"])


def test_gap_cutoff_masks_pairs(api, c1):
    ds = c1.dataset
    params = _params(c1)
    cut = float(np.quantile(ds.gapfrequency, 0.7))
    total, Z, u = api.computestructureintegratedlikelihood(ds, params, c1.W, gapcutoff=cut, return_unpaired=True)
    rp = mr.getparams(c1.params15, ds.branchlengths)
    p, _ = mr.pair_loglik(ds.tree_arrays(), ds.masks, rp, c1.W)
    p = co.maskgapped(p, ds.gapfrequency, cut)
    uref, _ = mr.unpaired_loglik(ds.tree_arrays(), ds.masks, rp)
    Zref = co.inside(uref, p)[0, 0, ds.numcols - 1]
    assert abs(Z - Zref) <= REL * abs(Zref)
    np.testing.assert_allclose(u, uref, rtol=1e-11)


def test_native_kernels_ran(api, c1):
    ctx = api.get_context()
    api.computestructureintegratedlikelihood(c1.dataset, _params(c1), c1.W)
    assert ctx.last_launches() > 10
    st = ctx.dataset(c1.dataset, c1.W).stats()
    assert st["band_pairs"] == 7140 and st["unique_root_pairs"] <= 7140
    assert 0 < st["executed_updates_per_category"] <= st["naive_updates_per_category"]


def test_invalid_model_is_rejected(api, c1):
    from messi_gb300._lib import MessiError
    params = _params(c1)
    params.freqs = np.array([0.5, 0.5, 0.1, -0.1])
    with pytest.raises(MessiError):
        api.felsensteincuda(c1.dataset, params, None, c1.W)
