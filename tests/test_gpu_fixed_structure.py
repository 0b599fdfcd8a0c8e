"""Fixed-structure likelihood (messi_structure_likelihood): the usecuda
branch of computemodellikelihood, src/FARCE.jl:2480-2485, against the FP64
oracle (relative 1e-6) and against the band path (the same per-pattern
arithmetic, so the pair values agree to rounding)."""
import numpy as np
import pytest

from oracle import model_ref as mr

pytestmark = pytest.mark.gpu

REL = 1e-6


def _one_based(partner0):
    return np.where(np.asarray(partner0) >= 0, np.asarray(partner0) + 1, 0).astype(np.int64)


def test_structure_likelihood_matches_oracle_and_band_path(c1):
    from messi_gb300 import api
    from messi_gb300 import model as M
    ds = c1.dataset
    L = ds.numcols
    params = M.getparams(c1.params15, ds.branchlengths)
    paired = _one_based(c1.paired)
    assert np.count_nonzero(paired) > 10
    total, pairll, u = api._structure_call(ds, params, paired, api.get_context())
    rp = mr.getparams(c1.params15, ds.branchlengths)
    mask = np.zeros((L, L), np.uint8)
    for x in range(L):
        if paired[x] > x + 1:
            mask[x, paired[x] - 1] = mask[paired[x] - 1, x] = 1
    pref, _ = mr.pair_loglik(ds.tree_arrays(), ds.masks, rp, L - 1, pairmask=mask)
    uref, _ = mr.unpaired_loglik(ds.tree_arrays(), ds.masks, rp)
    ref_total = 0.0
    for x in range(L):
        if paired[x] == 0:
            ref_total += uref[x]
            assert abs(u[x] - uref[x]) <= 1e-11 * abs(uref[x])
            assert pairll[x] == 0.0
        else:
            assert u[x] == 0.0
            if paired[x] > x + 1:
                y = paired[x] - 1
                ref_total += pref[x, y]
                assert abs(pairll[x] - pref[x, y]) <= REL * abs(pref[x, y])
    assert abs(total - ref_total) <= REL * abs(ref_total)
    # the band path computes the same pair values
    mat, _ = api.felsensteincuda(ds, params, None, L - 1)
    for x in range(L):
        if paired[x] > x + 1:
            assert abs(pairll[x] - mat[x, paired[x] - 1]) <= 1e-12 * abs(mat[x, paired[x] - 1])
    assert abs(api.felsensteincudapaired(ds, paired, params) - pairll.sum()) <= 1e-12 * abs(pairll.sum())
    prior = M.computeprior(params)
    assert abs(api.computemodellikelihood(None, ds, params, paired) - (prior + total)) <= 1e-12 * abs(total)
    u2 = api.computeunpairedlikelihoods(ds, params, None, None, paired)
    np.testing.assert_array_equal(u2, u)


def test_empty_and_invalid_structures(c1):
    from messi_gb300 import api
    from messi_gb300 import model as M
    from messi_gb300._lib import MessiError
    ds = c1.dataset
    params = M.getparams(c1.params15, ds.branchlengths)
    L = ds.numcols
    none = np.zeros(L, np.int64)
    total, pairll, u = api._structure_call(ds, params, none, api.get_context())
    np.testing.assert_allclose(total, api.computeunpairedlikelihoods(ds, params).sum(), rtol=1e-12)
    assert api.felsensteincudapaired(ds, none, params) == 0.0
    bad = none.copy()
    bad[3] = 9  # partner of column 4 is column 9, but column 9 points nowhere
    with pytest.raises(MessiError):
        api._structure_call(ds, params, bad, api.get_context())
