"""Site-rate conditionals (felsensteinposteriorsiterateconditionalscuda,
src/FelsensteinCUDA.jl:518-717) against the FP64 oracle: relative 1e-6."""
import numpy as np
import pytest

from oracle import c_oracle as co
from oracle import model_ref as mr

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("W", [119, 30])
def test_siterate_conditionals_match_oracle(c1, W):
    from messi_gb300 import api
    from messi_gb300 import model as M
    ds = c1.dataset
    rp = mr.getparams(c1.params15, ds.branchlengths)
    u, _ = mr.unpaired_loglik(ds.tree_arrays(), ds.masks, rp)
    p, _ = mr.pair_loglik(ds.tree_arrays(), ds.masks, rp, W)
    ins = co.inside(u, p)
    single, pair = co.basepairprobs(ins, co.outside(ins, u, p), u, p)
    ref = mr.siterate_conditionals(ds.tree_arrays(), ds.masks, rp, W, single, pair)
    got = api.felsensteinposteriorsiterateconditionalscuda(single, pair, ds, M.getparams(c1.params15, ds.branchlengths),
                                                             None, W)
    assert got.shape == ref.shape == (3, ds.numcols)
    fin = np.isfinite(ref)
    assert np.array_equal(fin, np.isfinite(got))
    err = np.abs(got[fin] - ref[fin]) / np.maximum(np.abs(ref[fin]), 1.0)
    assert err.max() <= 1e-6, err.max()
