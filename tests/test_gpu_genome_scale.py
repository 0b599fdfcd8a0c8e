"""Genome-scale parity: 30 sequences x 9,000 columns, pair span <= 800.

At this size the dense FP64 oracle is out of reach (O(L^3) inside, 7.2e6
pairs x 45 categories of FP64 pruning), so parity is checked through
  * the pair likelihoods of sampled row blocks against the FP64 oracle,
  * the unpaired column likelihoods of every column,
  * Z of the GPU inside pass against the FP64 banded inside pass run on the
    same (u, p) inputs,
  * size-independent properties: symmetry and the finite pattern of the
    matrix (band minus all-gap columns).
Tolerance: relative 1e-6 on every log-likelihood.
"""
import numpy as np
import pytest

from oracle import c_oracle as co
from oracle import model_ref as mr

pytestmark = pytest.mark.gpu

REL = 1e-6


@pytest.fixture(scope="module")
def c4():
    from messi_gb300 import synth
    return synth.make_workload("c4", seed=1)


def test_genome_scale_pairs_unpaired_and_Z(c4):
    from messi_gb300 import api
    from messi_gb300 import model as M

    ds = c4.dataset
    L, W = ds.numcols, c4.W
    params = M.getparams(c4.params15, ds.branchlengths)
    rp = mr.getparams(c4.params15, ds.branchlengths)

    mat, _ = api.felsensteincuda(ds, params, None, W)
    assert mat.shape == (L, L)

    # band pattern and symmetry over the whole matrix
    fin = np.isfinite(mat)
    i, j = np.nonzero(fin)
    assert np.all(i != j) and np.all(np.abs(i - j) <= W)
    assert fin.sum() == 2 * sum(L - d for d in range(1, W + 1))
    assert np.array_equal(mat[i, j], mat[j, i])

    # sampled row blocks against the FP64 oracle
    for x0, x1 in ((0, 4), (4400, 4404), (8990, 9000)):
        ref, _ = mr.pair_loglik(ds.tree_arrays(), ds.masks, rp, W, rows=(x0, x1))
        blk = ref[x0:x1]
        g = mat[x0:x1]
        upper = np.arange(L)[None, :] > np.arange(x0, x1)[:, None]
        ok = np.isfinite(blk) & upper
        assert ok.sum() > 0
        assert np.array_equal(ok, np.isfinite(g) & upper)
        err = np.abs(g[ok] - blk[ok]) / np.abs(blk[ok])
        assert err.max() <= REL, f"rows {x0}:{x1} max relative error {err.max():.3e}"

    u = api.computeunpairedlikelihoods(ds, params)
    uref, _ = mr.unpaired_loglik(ds.tree_arrays(), ds.masks, rp)
    np.testing.assert_allclose(u, uref, rtol=1e-11)

    api.maskgapped(mat, ds.gapfrequency, 1.0, -np.inf)
    Z = api.computeinsideKH99(u, mat)
    Zref = co.inside_banded_Z(u, mat, W)
    assert abs(Z - Zref) <= REL * abs(Zref), (Z, Zref)

    # the fused call (pairs, unpaired, mask, inside, prior) agrees too
    total = api.computestructureintegratedlikelihood(ds, params, W)
    prior = M.computeprior(params)
    assert abs(total - (prior + Zref)) <= REL * abs(Zref)
