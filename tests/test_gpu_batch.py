"""Batched evaluation of many alignments (messi_batch_*) against the
single-alignment path and the FP64 oracle.

The batch prunes the tree levels of all alignments together and runs all
inside passes in one persistent launch; each alignment's arithmetic is the
same as in messi_likelihood, so Z must agree with the single-alignment call
to rounding (relative 1e-12) and with the oracle to the FP32 bar
(relative 1e-6).
"""
import numpy as np
import pytest

from oracle import model_ref as mr

pytestmark = pytest.mark.gpu

REL = 1e-6


@pytest.fixture(scope="module")
def batch_workloads():
    from messi_gb300 import synth
    return synth.make_batch("c3s", seed=1)


def _params(s):
    from messi_gb300 import model as M
    return M.getparams(s.params15, s.dataset.branchlengths)


def test_batch_equals_single_alignment_calls(batch_workloads):
    from messi_gb300 import api
    ws = batch_workloads
    b = api.Batch([w.dataset for w in ws])
    params = [_params(w) for w in ws]
    Z = b.likelihood(params)
    st = b.stats()
    assert st["nodes"] == sum(w.dataset.numnodes for w in ws)
    assert 0 < st["executed_updates_per_category"] <= st["naive_updates_per_category"]
    for w, p, z in zip(ws, params, Z):
        _, z1, _ = api.computestructureintegratedlikelihood(w.dataset, p, w.W, return_unpaired=True)
        assert abs(z - z1) <= 1e-12 * abs(z1), (w.dataset.numcols, z, z1)
    # a second evaluation reuses the arena and descriptors
    np.testing.assert_array_equal(b.likelihood(params), Z)


def test_batch_with_one_shared_model_and_gap_cutoff(batch_workloads):
    from messi_gb300 import api
    from messi_gb300 import model as M
    ws = batch_workloads[:10]
    b = api.Batch([w.dataset for w in ws], maxbasepairdistance=[max(1, w.dataset.numcols // 3) for w in ws])
    shared = [M.getparams(ws[0].params15, w.dataset.branchlengths) for w in ws]
    cut = 0.08
    Z = b.likelihood(shared, gapcutoff=cut)
    for w, p, z in zip(ws, shared, Z):
        _, z1, _ = api.computestructureintegratedlikelihood(w.dataset, p, max(1, w.dataset.numcols // 3),
                                                            gapcutoff=cut, return_unpaired=True)
        assert abs(z - z1) <= 1e-12 * abs(z1)


def test_batch_matches_oracle(batch_workloads):
    from messi_gb300 import api
    ws = [w for w in batch_workloads if w.dataset.numcols <= 90][:4]
    assert ws
    b = api.Batch([w.dataset for w in ws])
    totals = api.computestructureintegratedlikelihoods([w.dataset for w in ws], [_params(w) for w in ws], batch=b)
    for w, tot in zip(ws, totals):
        ds = w.dataset
        ref, _ = mr.structure_integrated_likelihood(ds.tree_arrays(), ds.masks, ds.gapfrequency, w.params15, w.W)
        assert abs(tot - ref) <= REL * abs(ref), (ds.numcols, tot, ref)
