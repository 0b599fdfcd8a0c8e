"""Parity on the benchmarked workloads, against the FP64 oracle chain.

The performance figures rest on these configurations, so each one's error
against the FP64 restatement of the reference's CPU path is asserted and
printed (lines starting with PARITY; run with -s to see them):

  c2  64 seqs x 1,000 nt, span 500 (the bench line's workload, seed 1):
      every one of the 374,750 pair log-likelihoods, the unpaired column
      log-likelihoods, Z of the fused evaluation (messi_likelihood) against
      the FP64 chain unpaired -> pairs -> maskgapped -> inside, and the
      base-pairing posteriors of the GPU chain against the FP64 chain.
  c3  256 alignments, L ~ U(80, 1500), W = L - 1: Z of every batch member
      against the FP64 inside pass on that member's GPU pair matrix, every
      member's unpaired columns, and two rows of pairs per member against the
      FP64 pruning (the full FP64 pair matrices of all 256 would take most of
      an hour on the host).
  c4  30 seqs x 9,000 nt, span 800: the whole FP64 chain (7.2e6 pairs) and
      the posteriors from the banded FP64 chain (the dense one is O(L^3)).

Tolerances: log-likelihoods (pairs, unpaired, Z) relative 1e-6 (the bar the
FP32 path is held to); posteriors absolute 1e-4, and 3e-4 at genome scale.
Inside/outside cells are FP32 log-odds, each carrying ~|x| 2^-24; the S cells
of the last column (the outside of S(i, L-1) and its inside) hold the
log-odds of the whole prefix or suffix of the alignment, which at 9,000
columns reaches thousands of nats (ulp ~2.4e-4 at 4,000), and the posteriors
of cells whose outside sums reach that column inherit it: c4 measures
1.55e-4 with the GPU's own scores as with the FP64 ones.
Reference: src/FARCE.jl:2322-2345 (the likelihood),
src/InsideOutsideAlgorithm.jl:486-533 (the posteriors).
"""
import numpy as np
import pytest

from oracle import c_oracle as co
from oracle import model_ref as mr

pytestmark = pytest.mark.gpu

REL = 1e-6
POST_TOL = 1e-4
POST_TOL_GENOME = 3e-4


def _rel_err(got, ref):
    fin = np.isfinite(ref)
    assert np.array_equal(fin, np.isfinite(got)), "finite pattern differs"
    if not fin.any():
        return 0.0
    return float((np.abs(got[fin] - ref[fin]) / np.maximum(np.abs(ref[fin]), 1.0)).max())


def _post_err(single, pair, s_ref, up_ref, lo_ref, W):
    up, lo = co.band_of(pair, W)
    e = max(float(np.abs(single - s_ref).max()), float(np.abs(up - up_ref).max()), float(np.abs(lo - lo_ref).max()))
    # nothing outside the band
    L = len(single)
    i, j = np.nonzero(pair)
    assert np.all(np.abs(i - j) <= W) and np.all(i != j)
    return e


@pytest.fixture(scope="module")
def c2():
    from messi_gb300 import synth
    return synth.make_workload("c2", seed=1)


def test_c2_pairs_Z_and_posteriors_against_fp64_chain(c2):
    from messi_gb300 import api
    from messi_gb300 import model as M
    ds = c2.dataset
    L, W = ds.numcols, c2.W
    params = M.getparams(c2.params15, ds.branchlengths)
    rp = mr.getparams(c2.params15, ds.branchlengths)
    tree = ds.tree_arrays()

    # FP64 chain
    u_ref, _ = mr.unpaired_loglik(tree, ds.masks, rp)
    p_ref, _ = mr.pair_loglik(tree, ds.masks, rp, W)
    pm_ref = co.maskgapped(p_ref, ds.gapfrequency, 1.0)
    Z_ref, s_ref, up_ref, lo_ref = co.posteriors_banded(u_ref, pm_ref, W)
    total_ref = mr.computeprior(rp) + Z_ref

    # GPU: the reference-facing calls
    u = api.computeunpairedlikelihoods(ds, params)
    mat, _ = api.felsensteincuda(ds, params, None, W)
    e_pair = _rel_err(mat, p_ref)
    fin = np.isfinite(p_ref)
    d = mat[fin] - p_ref[fin]
    print(f"\nPARITY c2 pairs: signed error mean {d.mean():.3e}, sd {d.std():.3e}, fraction below the FP64 value "
          f"{np.mean(d < 0):.3f}, max abs {np.abs(d).max():.3e} at |ref| {np.abs(p_ref[fin])[np.argmax(np.abs(d))]:.2f}")
    assert e_pair <= REL, f"c2 pair log-likelihoods: max relative error {e_pair:.3e}"
    np.testing.assert_allclose(u, u_ref, rtol=1e-11)
    assert int(np.isfinite(mat[np.triu_indices(L, 1)]).sum()) == 374750

    # GPU: the fused evaluation the bench times
    total = api.computestructureintegratedlikelihood(ds, params, W)
    e_Z = abs(total - total_ref) / abs(total_ref)
    assert e_Z <= REL, f"c2 structure-integrated likelihood: relative error {e_Z:.3e} ({total} vs {total_ref})"

    # GPU posteriors: the whole FP32 chain against the FP64 chain, and the
    # inside/outside/posterior kernels alone on the GPU's own scores
    api.maskgapped(mat, ds.gapfrequency, 1.0, -np.inf)
    Zg, single, pair = api.computeposteriors(u, mat)
    e_post = _post_err(single, pair, s_ref, up_ref, lo_ref, W)
    Z_same, s_same, up_same, lo_same = co.posteriors_banded(u, mat, W)
    e_post_same = _post_err(single, pair, s_same, up_same, lo_same, W)
    e_Zg = abs(Zg - Z_same) / abs(Z_same)
    print(f"\nPARITY c2: pairs max rel {e_pair:.3e}; Z (fused) rel {e_Z:.3e}; inside Z on GPU scores rel "
          f"{e_Zg:.3e}; posteriors max abs {e_post:.3e} (vs FP64 chain), {e_post_same:.3e} (same scores)")
    assert e_Zg <= REL
    assert e_post <= POST_TOL and e_post_same <= POST_TOL
    np.testing.assert_allclose(single + pair.sum(axis=1), 1.0, atol=1e-5)


def test_c3_every_batch_member_against_fp64(request):
    from messi_gb300 import api, synth
    from messi_gb300 import model as M
    ws = synth.make_batch("c3", seed=1)
    assert len(ws) == 256
    b = api.Batch([w.dataset for w in ws])
    params = [M.getparams(w.params15, w.dataset.branchlengths) for w in ws]
    Z = b.likelihood(params)
    b.close()
    worst_Z = worst_pair = 0.0
    rng = np.random.default_rng(3)
    for k, (w, prm, z) in enumerate(zip(ws, params, Z)):
        ds = w.dataset
        L = ds.numcols
        rp = mr.getparams(w.params15, ds.branchlengths)
        tree = ds.tree_arrays()
        u = api.computeunpairedlikelihoods(ds, prm)
        u_ref, _ = mr.unpaired_loglik(tree, ds.masks, rp)
        np.testing.assert_allclose(u, u_ref, rtol=1e-11)
        mat, _ = api.felsensteincuda(ds, prm, None, L - 1)
        # two rows of pairs against the FP64 pruning
        x0 = int(rng.integers(0, L - 2))
        blk, _ = mr.pair_loglik(tree, ds.masks, rp, L - 1, rows=(x0, x0 + 2))
        sel = np.arange(L)[None, :] > np.arange(x0, x0 + 2)[:, None]
        g, r = np.where(sel, mat[x0:x0 + 2], -np.inf), np.where(sel, blk[x0:x0 + 2], -np.inf)
        worst_pair = max(worst_pair, _rel_err(g, r))
        # Z of the batch member against the FP64 inside pass on its GPU scores
        api.maskgapped(mat, ds.gapfrequency, 1.0, -np.inf)
        z_ref = co.inside_banded_Z(u, mat, L - 1)
        worst_Z = max(worst_Z, abs(z - z_ref) / abs(z_ref))
    print(f"\nPARITY c3: 256 members; Z max rel {worst_Z:.3e} (batch vs FP64 inside on GPU scores); "
          f"sampled pairs max rel {worst_pair:.3e}")
    assert worst_Z <= REL and worst_pair <= REL


def test_c4_fp64_chain_and_posteriors():
    from messi_gb300 import api, synth
    from messi_gb300 import model as M
    c4 = synth.make_workload("c4", seed=1)
    ds = c4.dataset
    L, W = ds.numcols, c4.W
    params = M.getparams(c4.params15, ds.branchlengths)
    rp = mr.getparams(c4.params15, ds.branchlengths)
    tree = ds.tree_arrays()
    # the whole FP64 chain
    u_ref, _ = mr.unpaired_loglik(tree, ds.masks, rp)
    p_ref, _ = mr.pair_loglik(tree, ds.masks, rp, W)
    pm_ref = co.maskgapped(p_ref, ds.gapfrequency, 1.0)
    del p_ref
    Z_ref, s_ref, up_ref, lo_ref = co.posteriors_banded(u_ref, pm_ref, W)
    total_ref = mr.computeprior(rp) + Z_ref
    total = api.computestructureintegratedlikelihood(ds, params, W)
    e_Z = abs(total - total_ref) / abs(total_ref)
    assert e_Z <= REL, f"c4 structure-integrated likelihood: relative error {e_Z:.3e}"
    mat, _ = api.felsensteincuda(ds, params, None, W)
    api.maskgapped(mat, ds.gapfrequency, 1.0, -np.inf)
    e_pair = _rel_err(mat, pm_ref)
    del pm_ref
    assert e_pair <= REL, f"c4 pair log-likelihoods: max relative error {e_pair:.3e}"
    u = api.computeunpairedlikelihoods(ds, params)
    Zg, single, pair = api.computeposteriors(u, mat, maxspan=W)
    e_post = _post_err(single, pair, s_ref, up_ref, lo_ref, W)
    del s_ref, up_ref, lo_ref
    _, s_same, up_same, lo_same = co.posteriors_banded(u, mat, W)
    e_post_same = _post_err(single, pair, s_same, up_same, lo_same, W)
    print(f"\nPARITY c4: pairs max rel {e_pair:.3e}; Z (fused) rel {e_Z:.3e}; posteriors max abs {e_post:.3e} "
          f"(vs FP64 chain), {e_post_same:.3e} (same scores)")
    assert e_post <= POST_TOL_GENOME and e_post_same <= POST_TOL_GENOME
