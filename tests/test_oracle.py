"""Pins the FP64 CPU oracle with derived known-answer tests.

The reference has no test suite or golden vectors, so the oracle is pinned by
identities of the model and the grammar and by an independent numpy
restatement (oracle/oracle_np.py).
"""
import numpy as np
import pytest
from scipy.linalg import expm

from oracle import c_oracle as co
from oracle import model_ref as mr
from oracle import oracle_np as onp


def _rand_model(seed):
    rng = np.random.default_rng(seed)
    pi = rng.dirichlet([5, 5, 5, 5])
    q = rng.uniform(0.2, 5.0, 6)
    lam = rng.uniform(1.0, 5.0, 3)
    return pi, q, lam


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_rate_matrices_match_numpy_and_are_reversible(seed):
    pi, q, lam = _rand_model(seed)
    Q4 = co.gtr(q, pi)
    np.testing.assert_allclose(Q4, onp.gtr(q, pi), rtol=1e-14, atol=1e-14)
    np.testing.assert_allclose(Q4.sum(axis=1), 0, atol=1e-13)
    Q = co.muse(lam[0], lam[1], lam[2], q, pi, 0.7, 1.9)
    np.testing.assert_allclose(Q, onp.muse(lam[0], lam[1], lam[2], q, pi, 0.7, 1.9), rtol=1e-13, atol=1e-13)
    np.testing.assert_allclose(Q.sum(axis=1), 0, atol=1e-12)
    f = co.musefreqs(pi, *lam)
    assert abs(f.sum() - 1) < 1e-14
    np.testing.assert_allclose(f, onp.musefreqs(pi, *lam), rtol=1e-13)
    # stationarity and detailed balance
    np.testing.assert_allclose(f @ Q, 0, atol=1e-12)
    D = f[:, None] * Q
    np.testing.assert_allclose(D, D.T, atol=1e-13)


@pytest.mark.parametrize("seed", [0, 3])
def test_transition_matrices_match_expm(seed):
    pi, q, lam = _rand_model(seed)
    Q = co.muse(lam[0], lam[1], lam[2], q, pi, 1.3, 0.4)
    f = co.musefreqs(pi, *lam)
    bl = np.array([0.0, 0.0, 0.01, 0.1, 0.5, 2.0])
    P = co.transition_matrices(Q, f, bl)
    assert np.all(P[0] == 0)                           # root: unused, zeros
    np.testing.assert_allclose(P[1], np.eye(16))       # zero branch: identity
    for k in range(2, len(bl)):
        E = expm(Q * bl[k])
        E[E <= 0] = 1e-50
        np.testing.assert_allclose(P[k], E, rtol=1e-10, atol=1e-13)
        np.testing.assert_allclose(P[k].sum(axis=1), 1, atol=1e-12)


def test_logsumexp_matches_reference_semantics():
    assert co.logsumexp(-np.inf, 3.0) == 3.0
    assert co.logsumexp(2.0, -np.inf) == 2.0
    assert abs(co.logsumexp(1.0, 2.0) - np.logaddexp(1.0, 2.0)) < 1e-15


def test_subcolumnrefs_are_first_occurrences(tiny):
    ds = tiny.dataset
    refs = co.subcolumnrefs(ds.children, ds.seqindex, ds.masks)
    # leaves: same mask <=> same ref; refs point at the first such column
    for v in range(ds.numnodes):
        if ds.children[v, 0] < 0:
            row = ds.masks[ds.seqindex[v]]
            for x in range(ds.numcols):
                assert refs[v, x] == int(np.argmax(row == row[x]))
    # root: columns equal across all sequences <=> same ref
    for x in range(ds.numcols):
        for y in range(ds.numcols):
            same = bool(np.all(ds.masks[:, x] == ds.masks[:, y]))
            assert (refs[0, x] == refs[0, y]) == same


def test_pair_likelihoods_match_plain_recursion(tiny):
    ds = tiny.dataset
    rp = mr.getparams(tiny.params15, ds.branchlengths)
    P, pi16, logw, *_ = mr.pair_categories(rp)
    out, _ = co.pair_matrix(ds.children, ds.seqindex, ds.masks, P, pi16, logw, tiny.W)
    # independent recursion with expm-built P for every category
    Pnp, pinp, lw = [], [], []
    for a in range(3):
        for b in range(3):
            for k in range(5):
                l3 = [rp.lambdaratesGC[k] + 1, rp.lambdaratesAT[k] + 1, rp.lambdaratesGT[k] + 1]
                Q = onp.muse(*l3, rp.q, rp.freqs, rp.siteRates[a], rp.siteRates[b])
                Pnp.append(onp.transition_matrices(Q, ds.branchlengths))
                pinp.append(onp.musefreqs(rp.freqs, *l3))
    for (x, y) in [(0, 1), (0, 13), (3, 9), (5, 6), (2, 11)]:
        lls = [onp.prune_column_pair(ds.children, ds.seqindex, ds.masks, Pnp[c], pinp[c], x, y) for c in range(45)]
        ref = -np.inf
        for c in range(45):
            ref = np.logaddexp(ref, logw[c] + lls[c])
        assert abs(out[x, y] - ref) < 1e-10 * abs(ref)
        assert out[y, x] == out[x, y]
    assert np.all(np.isneginf(np.diag(out)))


def test_unpaired_matches_plain_recursion(tiny):
    ds = tiny.dataset
    rp = mr.getparams(tiny.params15, ds.branchlengths)
    u, ubs = mr.unpaired_loglik(ds.tree_arrays(), ds.masks, rp)
    for x in range(ds.numcols):
        vals = []
        for r in rp.siteRates:
            Pn = onp.transition_matrices(onp.gtr(rp.q, rp.freqs) * r, ds.branchlengths)
            vals.append(onp.prune_column_pair(ds.children, ds.seqindex, ds.masks, Pn, rp.freqs, x))
        ref = np.logaddexp.reduce(np.log(1 / 3) + np.array(vals))
        assert abs(u[x] - ref) < 1e-11 * abs(ref)


def test_lambda_one_factorises(tiny):
    """lambda = 1: the 16-state pair model is the product of two unpaired
    columns (the identity src/FARCE.jl:1891-1901 relies on)."""
    ds = tiny.dataset
    rp = mr.getparams(tiny.params15, ds.branchlengths)
    u, ubs = mr.unpaired_loglik(ds.tree_arrays(), ds.masks, rp)
    a, b = mr.pair_loglik(ds.tree_arrays(), ds.masks, rp, tiny.W)
    c, _ = mr.pair_loglik(ds.tree_arrays(), ds.masks, rp, tiny.W, lambda1_factorised=True, u_by_site=ubs)
    fin = np.isfinite(a)
    np.testing.assert_allclose(a[fin], c[fin], rtol=1e-11)
    # category with lambda = 1 directly: 16-state likelihood == u1[x] + u2[y]
    P, pi16, logw, lam, l1, s1, s2 = mr.pair_categories(rp)
    k = int(np.where(l1 == 1)[0][0])
    one, _ = co.pair_matrix(ds.children, ds.seqindex, ds.masks, P[k:k + 1], pi16[k:k + 1], np.zeros(1), tiny.W)
    for (x, y) in [(0, 5), (1, 2), (4, 13)]:
        assert abs(one[x, y] - (ubs[s1[k], x] + ubs[s2[k], y])) < 1e-10 * abs(one[x, y])


def test_per_lambda_conditionals_mix_to_total(tiny):
    ds = tiny.dataset
    rp = mr.getparams(tiny.params15, ds.branchlengths)
    tot, per = mr.pair_loglik(ds.tree_arrays(), ds.masks, rp, tiny.W, per_lambda=True)
    fin = np.isfinite(tot)
    np.testing.assert_allclose(np.logaddexp.reduce(per, axis=0)[fin], tot[fin], rtol=1e-12)


def test_band_and_mask_select_pairs(tiny):
    ds = tiny.dataset
    rp = mr.getparams(tiny.params15, ds.branchlengths)
    full, _ = mr.pair_loglik(ds.tree_arrays(), ds.masks, rp, 13)
    band, _ = mr.pair_loglik(ds.tree_arrays(), ds.masks, rp, 4)
    L = ds.numcols
    for x in range(L):
        for y in range(L):
            if x != y and abs(x - y) <= 4:
                assert band[x, y] == full[x, y]
            else:
                assert np.isneginf(band[x, y])
    mask = np.ones((L, L), np.uint8)
    mask[2, 7] = mask[7, 2] = 0
    m, _ = mr.pair_loglik(ds.tree_arrays(), ds.masks, rp, 13, pairmask=mask)
    assert np.isneginf(m[2, 7]) and m[2, 8] == full[2, 8]


def test_inside_closed_form_when_no_pairs():
    rng = np.random.default_rng(5)
    L = 30
    u = rng.uniform(-40, -5, L)
    p = np.full((L, L), -np.inf)
    Z = co.inside(u, p)[0, 0, L - 1]
    r = co.kh99_logprobs()
    assert abs(Z - (u.sum() + (L - 1) * (r[0] + r[5]) + r[1])) < 1e-10 * abs(Z)


@pytest.mark.parametrize("L", [1, 2, 5, 8, 10])
def test_inside_equals_brute_force_enumeration(L):
    rng = np.random.default_rng(L)
    u = rng.uniform(-12, -2, L)
    p = rng.uniform(-25, -2, (L, L))
    p = np.triu(p, 1) + np.triu(p, 1).T
    ins = co.inside(u, p)
    assert abs(ins[0, 0, L - 1] - onp.brute_force_Z(u, p)) < 1e-10 * max(1.0, abs(ins[0, 0, L - 1]))
    np.testing.assert_allclose(ins[np.isfinite(ins)], onp.inside(u, p)[np.isfinite(ins)], rtol=1e-12)


@pytest.mark.parametrize("L", [6, 9])
def test_posteriors_equal_brute_force(L):
    rng = np.random.default_rng(100 + L)
    u = rng.uniform(-10, -4, L)
    p = rng.uniform(-16, -4, (L, L))
    p = np.triu(p, 1) + np.triu(p, 1).T
    ins = co.inside(u, p)
    outs = co.outside(ins, u, p)
    single, pair = co.basepairprobs(ins, outs, u, p)
    bs, bp = onp.brute_force_posteriors(u, p)
    np.testing.assert_allclose(single, bs, atol=1e-12)
    np.testing.assert_allclose(pair, bp, atol=1e-12)
    np.testing.assert_allclose(single + pair.sum(axis=1), 1.0, atol=1e-12)


def test_outside_inside_consistency(c1):
    """sum over the three nonterminals of inside x outside on the diagonal
    reproduces Z for every column (each column is emitted once)."""
    ds = c1.dataset
    _, info = mr.structure_integrated_likelihood(ds.tree_arrays(), ds.masks, ds.gapfrequency, c1.params15, c1.W)
    u, p, ins, Z = info["u"], info["p"], info["inside"], info["Z"]
    outs = co.outside(ins, u, p)
    single, pair = co.basepairprobs(ins, outs, u, p)
    np.testing.assert_allclose(single + pair.sum(axis=1), 1.0, atol=1e-10)
    assert abs(outs[0, 0, len(u) - 1]) == 0.0


def test_maskgapped():
    L = 5
    p = np.zeros((L, L))
    gf = np.array([0.0, 1.0, 0.2, 1.0, 0.0])
    m = co.maskgapped(p, gf, 1.0)
    assert np.isneginf(m[1, 0]) and np.isneginf(m[4, 3]) and m[0, 2] == 0.0


@pytest.mark.parametrize("L,W", [(1, 3), (2, 1), (9, 3), (40, 7), (60, 59), (75, 20)])
def test_banded_inside_equals_dense(L, W):
    rng = np.random.default_rng(L * 7 + W)
    u = rng.uniform(-40, -5, L)
    p = np.full((L, L), -np.inf)
    for i in range(L):
        for j in range(i + 1, min(L, i + W + 1)):
            p[i, j] = p[j, i] = u[i] + u[j] + rng.normal(0, 5)
    Zd = co.inside(u, p)[0, 0, L - 1]
    Zb = co.inside_banded_Z(u, p, W)
    assert abs(Zd - Zb) <= 1e-12 * abs(Zd)


@pytest.mark.parametrize("L", [1, 2, 3, 6, 9])
def test_posterior_decoding_equals_brute_force(L):
    rng = np.random.default_rng(40 + L)
    p = rng.random((L, L)) ** 3
    p = np.triu(p, 1)
    p = p + p.T
    p /= max(1.0, p.sum(axis=1).max()) * 1.2
    single = 1.0 - p.sum(axis=1)
    e, s = co.posterior_decoding(single, p, 2.0)
    best, arg = onp.brute_force_decoding(single.astype(np.float32).astype(np.float64),
                                         p.astype(np.float32).astype(np.float64), 2.0)
    assert abs(float(e[0, L - 1]) - best) <= 1e-5 * max(1.0, abs(best))
    paired = co.posterior_traceback(s)
    got = tuple(sorted((i, paired[i] - 1) for i in range(L) if paired[i] - 1 > i))
    val = onp.decoding_score(got, single.astype(np.float32).astype(np.float64),
                             p.astype(np.float32).astype(np.float64), 2.0, 0, L - 1)
    assert abs(val - best) <= 1e-5 * max(1.0, abs(best))
    for i in range(L):
        if paired[i]:
            assert paired[paired[i] - 1] == i + 1


@pytest.mark.parametrize("L,W", [(1, 0), (2, 1), (9, 8), (40, 12), (60, 59), (130, 40), (200, 20)])
def test_banded_posterior_chain_matches_dense(L, W):
    """The banded inside -> outside -> posterior chain (used at genome scale)
    equals the dense chain when every pair beyond the band is -Inf."""
    rng = np.random.default_rng(L * 7 + W)
    u = rng.uniform(-80.0, -20.0, L)
    p = np.full((L, L), -np.inf)
    for i in range(L):
        j = np.arange(i + 1, min(L, i + W + 1))
        p[i, j] = u[i] + u[j] + rng.normal(-3.0, 4.0, len(j)) + (rng.random(len(j)) < 0.05) * 25.0
    p = np.maximum(p, p.T)
    ins = co.inside(u, p)
    outs = co.outside(ins, u, p)
    s_ref, p_ref = co.basepairprobs(ins, outs, u, p)
    Z, s, up, lo = co.posteriors_banded(u, p, W)
    up_ref, lo_ref = co.band_of(p_ref, W)
    assert abs(Z - ins[0, 0, L - 1]) <= 1e-12 * max(1.0, abs(Z))
    assert np.abs(s - s_ref).max() <= 1e-11
    assert np.abs(up - up_ref).max() <= 1e-11 and np.abs(lo - lo_ref).max() <= 1e-11
