"""Edge cases through the C ABI against the FP64 oracle: the smallest
alignments and trees, ambiguity codes, all-gap columns, a band of one,
constant columns, and invalid inputs that must be rejected with a status
(relative 1e-6 on every log-likelihood)."""
import ctypes

import numpy as np
import pytest

from oracle import c_oracle as co
from oracle import model_ref as mr

pytestmark = pytest.mark.gpu

REL = 1e-6


def _params(p15, ds):
    from messi_gb300 import model as M
    return M.getparams(p15, ds.branchlengths)


def _check_likelihood(ds, p15, W):
    from messi_gb300 import api
    total = api.computestructureintegratedlikelihood(ds, _params(p15, ds), W)
    ref, _ = mr.structure_integrated_likelihood(ds.tree_arrays(), ds.masks, ds.gapfrequency, p15, W)
    assert abs(total - ref) <= REL * abs(ref), (total, ref)
    return total


@pytest.fixture(scope="module")
def p15():
    from messi_gb300 import model as M
    return M.DEFAULT_PARAMS15.copy()


def test_one_column_and_two_columns(p15):
    from messi_gb300.dataset import Dataset
    newick = "(a:0.1,b:0.2,c:0.3);"
    one = Dataset.from_sequences(["a", "b", "c"], ["A", "G", "A"], newick)
    _check_likelihood(one, p15, 1)
    two = Dataset.from_sequences(["a", "b", "c"], ["AU", "GC", "AU"], newick)
    _check_likelihood(two, p15, 1)


def test_three_sequences_ambiguity_codes_and_gaps(p15):
    from messi_gb300.dataset import Dataset
    seqs = ["ACGURYN-ACGUAC", "RYKMSWBDHVN-GA", "acgu-ACGUACGUU"]
    ds = Dataset.from_sequences(["a", "b", "c"], seqs, "(a:0.1,b:0.2,c:0.3);")
    for W in (1, 5, 13):
        _check_likelihood(ds, p15, W)


def test_all_gap_and_constant_columns(p15):
    from messi_gb300.dataset import Dataset
    seqs = ["A-GGGCCC-UA", "A-GGACCC-UA", "A-GGGCCU-UA", "A-GAGCCC-UA"]
    ds = Dataset.from_sequences(["a", "b", "c", "d"], seqs, "(a:0.1,b:0.2,(c:0.05,d:0.07):0.1);")
    assert ds.gapfrequency[1] == 1.0 and ds.gapfrequency[8] == 1.0
    _check_likelihood(ds, p15, 10)


def test_zero_branch_lengths_and_caterpillar_tree(p15):
    from messi_gb300.dataset import Dataset
    newick = "(a:0.0,(b:0.1,(c:0.0,(d:0.2,(e:0.05,f:0.3):0.0):0.1):0.2):0.0,g:0.4);"
    rng = np.random.default_rng(3)
    seqs = ["".join(rng.choice(list("ACGU"), 24)) for _ in range(7)]
    ds = Dataset.from_sequences(list("abcdefg"), seqs, newick)
    _check_likelihood(ds, p15, 23)


def test_inside_degenerate_scores():
    from messi_gb300 import api
    L = 6
    u = np.full(L, -5.0)
    p = np.full((L, L), -np.inf)
    # no pair possible: closed form of the grammar
    r = co.kh99_logprobs()
    Z = api.computeinsideKH99(u, p)
    assert abs(Z - (u.sum() + (L - 1) * (r[0] + r[5]) + r[1])) <= REL * abs(Z)
    # a single possible pair
    p[0, 5] = p[5, 0] = -3.0
    Z = api.computeinsideKH99(u, p)
    Zref = co.inside(u, p)[0, 0, L - 1]
    assert abs(Z - Zref) <= REL * abs(Zref)


def test_invalid_inputs_are_rejected(c1, p15):
    from messi_gb300 import api
    from messi_gb300._lib import MessiError
    ds = c1.dataset
    prm = _params(p15, ds)
    prm.branchlengths = prm.branchlengths.copy()
    prm.branchlengths[3] = -1.0
    with pytest.raises(MessiError):
        api.felsensteincuda(ds, prm, None, 10)
    with pytest.raises(MessiError):
        api.computeposteriordecodingcuda(np.zeros(0), np.zeros((0, 0)))
    bad = np.zeros(ds.numcols, np.int64)
    bad[0] = ds.numcols + 5
    with pytest.raises(MessiError):
        api.felsensteincudapaired(ds, bad, _params(p15, ds))


def test_bounded_wait_gives_up_and_context_stays_usable():
    """A grid barrier that one CTA never reaches: the waiting CTA gives up
    after a bounded spin, the host reads MESSI_ETIMEOUT, and the context
    keeps working (no fault, no unbounded wait)."""
    from messi_gb300 import api
    from messi_gb300._lib import MESSI_ETIMEOUT
    ctx = api.get_context()
    assert ctx.selftest_bounded_wait() == MESSI_ETIMEOUT
    L = 12
    u = np.full(L, -5.0)
    p = np.full((L, L), -np.inf)
    p[0, 11] = p[11, 0] = -3.0
    Z = api.computeinsideKH99(u, p, ctx=ctx)
    Zref = co.inside(u, p)[0, 0, L - 1]
    assert abs(Z - Zref) <= REL * abs(Zref)
    assert ctx.selftest_bounded_wait() == MESSI_ETIMEOUT


def test_wavefront_results_repeat_bit_for_bit():
    """The grid-barrier wavefronts (inside, outside, decoding) give the same
    bits on every run: a barrier that let a CTA read a cell before it was
    written would show up as run-to-run differences."""
    from messi_gb300 import api
    rng = np.random.default_rng(11)
    L, W = 400, 150
    u = rng.uniform(-30.0, -8.0, L)
    p = np.full((L, L), -np.inf)
    for i in range(L):
        for j in range(i + 1, min(L, i + W + 1)):
            p[i, j] = p[j, i] = u[i] + u[j] + rng.normal(-2.0, 3.0)
    Z0 = api.computeinsideKH99(u, p)
    post0 = api.computeposteriors(u, p)
    for _ in range(8):
        assert api.computeinsideKH99(u, p) == Z0
    for _ in range(3):
        post = api.computeposteriors(u, p)
        for a, b in zip(post, post0):
            np.testing.assert_array_equal(a, b)


def test_likelihood_graph_replay_equals_eager(c1, monkeypatch):
    """From the second identical call on, messi_likelihood replays a captured
    CUDA graph of its device work; the staged model is rewritten each call,
    so replays with new parameters must give exactly the eager results."""
    from messi_gb300 import api
    from messi_gb300 import model as M
    ds = c1.dataset
    rng = np.random.default_rng(5)
    p15s = []
    for _ in range(5):
        p = c1.params15.copy()
        p[0:3] *= np.exp(rng.normal(0, 0.1, 3))
        p[14] = min(0.9, max(0.1, p[14] + rng.normal(0, 0.05)))  # lambda-zero weight: the factorised term
        p15s.append(p)
    monkeypatch.setenv("MESSI_AUTOTUNE", "0")  # graphs from the second call (tuning calls run eagerly)
    ctx = api.Context(0)
    try:
        Zg = [api.computestructureintegratedlikelihood(ds, M.getparams(p, ds.branchlengths), c1.W, ctx=ctx)
              for p in p15s]
        replays = ctx.graph_replays()
    finally:
        ctx.close()
    monkeypatch.setenv("MESSI_GRAPHS", "0")
    ctx = api.Context(0)
    try:
        Ze = [api.computestructureintegratedlikelihood(ds, M.getparams(p, ds.branchlengths), c1.W, ctx=ctx)
              for p in p15s]
        assert ctx.graph_replays() == 0
    finally:
        ctx.close()
    assert Zg == Ze
    assert replays >= 3, replays


def test_likelihood_graph_dropped_with_its_dataset(c1, monkeypatch):
    """A captured likelihood graph holds its dataset's device pointers:
    destroying the dataset drops it, so a dataset created afterwards (which
    may reuse the host address) starts with eager calls and replays only its
    own capture, with the eager values."""
    from messi_gb300 import api
    from messi_gb300 import model as M
    ds = c1.dataset
    params = M.getparams(c1.params15, ds.branchlengths)
    monkeypatch.setenv("MESSI_AUTOTUNE", "0")
    ctx = api.Context(0)
    handles = []
    try:
        h1 = api.DatasetHandle(ctx, ds, c1.W)
        handles.append(h1)
        m = api.ModelArgs(params)

        def Z(h):
            z = ctypes.c_double()
            ctx.check(ctx.lib.messi_likelihood(ctx.handle, h.handle, ctypes.byref(m.struct), None, 1.0,
                                               ctypes.byref(z), None), "messi_likelihood")
            return z.value

        # the first call's scratch allocations change the key: capture from the third call
        first = [Z(h1) for _ in range(4)]
        r0 = ctx.graph_replays()
        assert r0 >= 1, r0
        h1.close()
        h2 = api.DatasetHandle(ctx, ds, c1.W)
        handles.append(h2)
        second = [Z(h2)]
        assert ctx.graph_replays() == r0  # no replay of the destroyed dataset's graph
        second += [Z(h2) for _ in range(3)]
        assert ctx.graph_replays() > r0
    finally:
        for h in handles:
            h.close()
        ctx.close()
    assert len(set(first + second)) == 1, first + second


@pytest.mark.parametrize("env", [{"MESSI_WAVE_THREADS": "1024"},
                                 {"MESSI_WAVE_THREADS": "256", "MESSI_WAVE_CTAS": "7"},
                                 {"MESSI_WAVE_CTAS": "1"}])
def test_inside_kernels_and_grids_bit_identical(env, monkeypatch):
    """Which kernel and grid run the inside pass changes only which warp
    computes a cell: the pipelined halves kernel (the default here, 256 and
    1,024 threads), the plain wavefront with 7 CTAs of 58 rows and with one
    CTA (rows beyond two per lane group computed whole) give the same bits."""
    from messi_gb300 import api
    rng = np.random.default_rng(12)
    L, W = 400, 150
    u = rng.uniform(-30.0, -8.0, L)
    p = np.full((L, L), -np.inf)
    for i in range(L):
        for j in range(i + 1, min(L, i + W + 1)):
            p[i, j] = p[j, i] = u[i] + u[j] + rng.normal(-2.0, 3.0)
    ctx = api.Context(0)
    try:
        T0 = api.computeinsideKH99(u, p, zonly=False, ctx=ctx)
        Z0 = api.computeinsideKH99(u, p, ctx=ctx)
        post0 = api.computeposteriors(u, p, ctx=ctx)
    finally:
        ctx.close()
    for k, v in env.items():
        monkeypatch.setenv(k, v)
    ctx = api.Context(0)
    try:
        T1 = api.computeinsideKH99(u, p, zonly=False, ctx=ctx)
        Z1 = api.computeinsideKH99(u, p, ctx=ctx)
        post1 = api.computeposteriors(u, p, ctx=ctx)
    finally:
        ctx.close()
    np.testing.assert_array_equal(T1, T0)
    assert Z1 == Z0
    for a, b in zip(post1, post0):
        np.testing.assert_array_equal(a, b)


def test_autotuner_tries_candidates_then_keeps_one_with_identical_results(c1):
    """The first evaluations of a dataset time candidate launch shapes (the
    pruning pipeline shape and the wavefront CTA size); then the chosen
    shapes are kept, the step is captured and replayed, and every call gives
    the same bits whatever shape ran it."""
    from messi_gb300 import api
    from messi_gb300 import model as M
    ds = c1.dataset
    params = M.getparams(c1.params15, ds.branchlengths)
    ctx = api.Context(0)
    try:
        shapes, Z = [], []
        for _ in range(8):
            Z.append(api.computestructureintegratedlikelihood(ds, params, c1.W, ctx=ctx))
            shapes.append(ctx.launch_shapes())
        assert len(set(Z)) == 1, Z
        # tuning calls cycle through the candidates (pruning shapes 0, 1, 2, 0;
        # CTA sizes automatic, 256, 512, 1024)
        assert [s["prune_shape"] for s in shapes[:4]] == [0, 1, 2, 0]
        assert [s["wave_threads"] for s in shapes[:4]] == [0, 256, 512, 1024]
        assert shapes[3]["tuned_workloads"] == 1
        assert all(s == shapes[4] for s in shapes[4:])
        assert ctx.graph_replays() >= 2
    finally:
        ctx.close()
