"""Categories with lambda = 1 (all three lambdas) are not pruned with 16
states: their pair likelihood is the product of the two unpaired columns
(the identity src/FARCE.jl:1891-1901 relies on), so the library adds
log(w) + u[x] + u[y] to the mixture instead.  These tests compare every
consumer of that shortcut against the oracle's full 16-state computation of
all 45 categories (relative 1e-6), and cover the models where nothing is
factorised (every lambda category at 1, a single lambda category) and a batch
whose model groups factorise differently."""
import numpy as np
import pytest

from oracle import model_ref as mr

pytestmark = pytest.mark.gpu

REL = 1e-6


def _close(got, ref, rel=REL):
    fin = np.isfinite(ref)
    assert np.array_equal(fin, np.isfinite(got)), "finite pattern differs"
    err = np.abs(got[fin] - ref[fin]) / np.maximum(np.abs(ref[fin]), 1.0)
    assert err.max() <= rel, f"max relative error {err.max():.3e}"


def _models(s, p15, lambdaCats=5):
    from messi_gb300 import model as M
    bl = s.dataset.branchlengths
    return M.getparams(p15, bl, lambdaCats=lambdaCats), mr.getparams(p15, bl, 3, lambdaCats)


@pytest.mark.parametrize("case", ["default", "all_lambda_one", "one_lambda_category"])
def test_pairs_and_per_lambda_against_full_oracle(c1, case):
    from messi_gb300 import api
    p15 = c1.params15.copy()
    lc = 5
    if case == "all_lambda_one":
        p15[0:3] = 1.0  # every lambda category has lambda = 1: nothing left to prune, nothing factorised
    if case == "one_lambda_category":
        lc = 1
    prm, rp = _models(c1, p15, lc)
    m = api.ModelArgs(prm)
    expected = {"default": 36, "all_lambda_one": 45, "one_lambda_category": 9}[case]
    assert m.pruned_categories() == expected
    ds = c1.dataset
    mat, per = api.felsensteincuda(ds, prm, None, c1.W, True)
    ref, refl = mr.pair_loglik(ds.tree_arrays(), ds.masks, rp, c1.W, per_lambda=True)
    _close(mat, ref)
    assert len(per) == len(refl)
    for k in range(len(per)):
        _close(per[k], refl[k])
    # the per-lambda mixtures mix to the total (both sums are FP32 over FP64 maxima)
    fin = np.isfinite(ref)
    np.testing.assert_allclose(np.logaddexp.reduce(np.array(per), axis=0)[fin], mat[fin], rtol=REL)


@pytest.mark.parametrize("case", ["default", "all_lambda_one"])
def test_likelihood_and_fixed_structure_against_full_oracle(c1, case):
    from messi_gb300 import api
    from messi_gb300 import model as M
    p15 = c1.params15.copy()
    if case == "all_lambda_one":
        p15[0:3] = 1.0
    prm, rp = _models(c1, p15)
    ds = c1.dataset
    ll = api.computestructureintegratedlikelihood(ds, prm, c1.W)
    ref, info = mr.structure_integrated_likelihood(ds.tree_arrays(), ds.masks, ds.gapfrequency, p15, c1.W)
    assert abs(ll - ref) <= REL * abs(ref), (ll, ref)
    # fixed structure: pairs of the generating structure
    L = ds.numcols
    paired = np.where(np.asarray(c1.paired) >= 0, np.asarray(c1.paired) + 1, 0).astype(np.int64)
    total = api.felsensteincudapaired(ds, paired, prm)
    ref_total = 0.0
    for x in range(L):
        if paired[x] > x + 1:
            ref_total += info["p"][x, paired[x] - 1]
    assert abs(total - ref_total) <= REL * abs(ref_total)
    whole = api.computemodellikelihood(None, ds, prm, paired)
    u = info["u"]
    ref_whole = M.computeprior(prm) + ref_total + sum(u[x] for x in range(L) if paired[x] == 0)
    assert abs(whole - ref_whole) <= REL * abs(ref_whole)


def test_batch_with_groups_that_factorise_differently():
    """Model groups with lambda = 1 categories and groups with every lambda at
    1: the batch keeps one category list for all and prunes all 45."""
    from messi_gb300 import api, synth
    ws = [w for w in synth.make_batch("c3s", seed=1) if w.dataset.numcols <= 90][:4]
    assert len(ws) >= 2
    prms, refs = [], []
    for i, w in enumerate(ws):
        p15 = w.params15.copy()
        if i % 2:
            p15[0:3] = 1.0
        prm, _ = _models(w, p15)
        prms.append(prm)
        ds = w.dataset
        _, info = mr.structure_integrated_likelihood(ds.tree_arrays(), ds.masks, ds.gapfrequency, p15, w.W)
        refs.append(info["Z"])
    b = api.Batch([w.dataset for w in ws])
    Z = b.likelihood(prms)
    for z, r in zip(Z, refs):
        assert abs(z - r) <= REL * abs(r), (z, r)
    # the same batch with one factorising model for all alignments
    prms = [_models(w, ws[0].params15)[0] for w in ws]
    Z = b.likelihood(prms)
    for w, p, z in zip(ws, prms, Z):
        _, z1, _ = api.computestructureintegratedlikelihood(w.dataset, p, w.W, return_unpaired=True)
        assert abs(z - z1) <= 1e-12 * abs(z1)
