"""Column-pattern compression on the device (messi_subcolumnrefs) against
the oracle's restatement of Dataset.subcolumnrefs (src/Dataset.jl:180-196):
bit-exact."""
import numpy as np
import pytest

from oracle import c_oracle as co

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("which", ["tiny", "c1", "c2"])
def test_subcolumnrefs_match_oracle(which, request):
    from messi_gb300 import api, synth
    s = synth.make_workload("c2", seed=1) if which == "c2" else request.getfixturevalue(which)
    ds = s.dataset
    got = api.subcolumnrefs(ds)
    ref = co.subcolumnrefs(ds.children, ds.seqindex, ds.masks)
    assert got.shape == (ds.numnodes, ds.numcols)
    np.testing.assert_array_equal(got, ref + 1)
