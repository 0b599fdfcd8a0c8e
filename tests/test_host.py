"""Host-side mirror of the reference interface (no GPU): ingest, rooting,
parameter discretisation, synthetic workloads."""
import numpy as np
import pytest

from messi_gb300 import model as M
from messi_gb300 import synth
from messi_gb300.dataset import Dataset, getnodelist, parse_newick, roottree, to_newick
from oracle import model_ref as mr


def test_newick_roundtrip_and_rooting():
    t = parse_newick("(a:0.1,(b:0.2,c:0.3)x:0.05,d:0.4);")
    assert [c.name for c in t.children] == ["a", "x", "d"]
    assert parse_newick(to_newick(t)).children[1].children[1].name == "c"
    r = roottree(t, 0)
    assert len(r.children) == 2
    assert r.children[0].name == "a" and abs(r.children[0].branchlength - 0.05) < 1e-15
    assert abs(r.children[1].branchlength - 0.05) < 1e-15  # old root gets the other half
    names = [n.name for n in getnodelist(r)]
    assert names == ["", "a", "", "x", "b", "c", "d"]


def test_dataset_masks_gaps_and_tree():
    fasta = ">a\nACGU-\n>b\nRYN-a\n>c\nAAAAA\n"
    ds = Dataset.from_fasta_newick(fasta, "(a:0.1,b:0.2,c:0.3);")
    assert ds.masks.tolist() == [[1, 2, 4, 8, 15], [5, 10, 15, 15, 1], [1, 1, 1, 1, 1]]
    # IUPAC codes, gaps and lower case all count as gaps (src/Dataset.jl:140-149)
    np.testing.assert_allclose(ds.gapfrequency, [1 / 3, 1 / 3, 1 / 3, 1 / 3, 2 / 3])
    assert ds.numnodes == 5 and ds.children[0].tolist() == [1, 2]
    assert ds.seqindex.tolist() == [-1, 0, -1, 1, 2]


def test_dataset_rejects_rooted_binary_newick():
    with pytest.raises(ValueError):
        Dataset.from_fasta_newick(">a\nA\n>b\nA\n>c\nA\n", "((a:0.1,b:0.2):0.1,c:0.3);")


def test_getparams_matches_oracle_restatement():
    bl = np.linspace(0, 1, 7)
    p = M.DEFAULT_PARAMS15.copy()
    p[:3] = [3.0, 2.5, 1.5]
    cp = M.getparams(p, bl)
    rp = mr.getparams(p, bl)
    np.testing.assert_allclose(cp.siteRates, rp.siteRates, rtol=1e-14)
    np.testing.assert_allclose(cp.lambdaratesGC, rp.lambdaratesGC, rtol=1e-14)
    np.testing.assert_allclose(cp.lambdaweightsGC, rp.lambdaweights)
    assert abs(M.computeprior(cp) - mr.computeprior(rp)) < 1e-12
    np.testing.assert_allclose(M.getparamsvector(cp), p)
    mps = M.getmusespecificparamsarray(cp)
    assert len(mps) == 5 and mps[0].lambdarate == 0.0 and abs(mps[0].prob - 0.5) < 1e-15


def test_single_lambda_category_and_factorised_count():
    """lambdaCats = 1 (src/FARCE.jl:609-657): one category with lambda = the
    lambda itself, weight 1; the library prunes categories with lambda != 1
    and factorises the rest unless nothing would be left."""
    from messi_gb300.api import ModelArgs
    bl = np.linspace(0, 1, 7)
    p = M.DEFAULT_PARAMS15.copy()
    p[:3] = [3.0, 2.5, 1.5]
    cp = M.getparams(p, bl, lambdaCats=1)
    rp = mr.getparams(p, bl, 3, 1)
    np.testing.assert_allclose(cp.lambdaratesGC, [2.0])
    np.testing.assert_allclose(cp.lambdaratesGT, [0.5])
    np.testing.assert_allclose(cp.lambdaweightsGC, [1.0])
    np.testing.assert_allclose(rp.lambdaratesAT, [1.5])
    np.testing.assert_allclose(rp.lambdaweights, [1.0])
    assert ModelArgs(cp).pruned_categories() == 9
    assert ModelArgs(M.getparams(p, bl)).pruned_categories() == 36
    p[:3] = 1.0
    assert ModelArgs(M.getparams(p, bl)).pruned_categories() == 45


def test_numpy_rate_matrices_match_oracle():
    from oracle import c_oracle as co
    pi = np.array([0.2, 0.3, 0.1, 0.4])
    q = np.array([1.0, 2.0, 0.5, 0.7, 3.0, 1.1])
    np.testing.assert_allclose(M.muse(2.0, 3.0, 1.5, q, pi, 0.4, 1.7), co.muse(2.0, 3.0, 1.5, q, pi, 0.4, 1.7),
                               rtol=1e-13, atol=1e-14)
    np.testing.assert_allclose(M.musefreqs(pi, 2.0, 3.0, 1.5), co.musefreqs(pi, 2.0, 3.0, 1.5), rtol=1e-13)


@pytest.mark.parametrize("name", ["c1"])
def test_synthetic_workload_shapes(name):
    s = synth.make_workload(name, seed=3)
    spec = synth.WORKLOADS[name]
    ds = s.dataset
    assert ds.numseqs == spec["numseqs"] and ds.numcols == spec["numcols"]
    assert ds.numnodes == 2 * ds.numseqs - 1
    frac = (s.paired >= 0).mean()
    assert abs(frac - spec["paired"]) < 0.05
    pairs = [(i, j) for i, j in enumerate(s.paired) if j > i]
    assert all(j - i <= spec["W"] and j - i >= 3 for i, j in pairs)
    for (i, j) in pairs:
        for (a, b) in pairs:
            assert not (i < a < j < b)
    assert 0.02 < ds.gapfrequency.mean() < 0.09
    # deterministic from the seed
    s2 = synth.make_workload(name, seed=3)
    assert s2.fasta == s.fasta and s2.newick == s.newick


def test_kh99_prior_matches_oracle():
    from messi_gb300.structures import calculateKH99prior
    from oracle import oracle_np as onp
    rng = np.random.default_rng(2)
    for L in (1, 2, 5, 9, 14):
        for s in list(onp._structures(0, L - 1))[:: max(1, len(list(onp._structures(0, L - 1))) // 7)]:
            paired0 = -np.ones(L, dtype=int)
            paired1 = np.zeros(L, dtype=int)
            for a, b in s:
                paired0[a], paired0[b] = b, a
                paired1[a], paired1[b] = b + 1, a + 1
            assert abs(calculateKH99prior(paired1) - onp.kh99_prior(paired0, L)) < 1e-12
