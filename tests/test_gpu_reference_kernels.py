"""Pins the FP64 oracle to the reference's own CUDA kernels.

src/cuda/felsenstein.cu and src/cuda/inside.cu, compiled unmodified for
sm_103a (oracle/_ref, ``make -C oracle ref``), run through a host harness
that replays the reference's launch sequences (oracle/ref_kernels.py).  The
reference kernels compute in FP32 (log space for the SCFG), so the tolerances
are FP32-sized; the same comparison is made for this library's kernels.
"""
import numpy as np
import pytest

from oracle import c_oracle as co
from oracle import model_ref as mr
from oracle import ref_kernels as rk

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not rk.available(), reason="reference cubins not built (make -C oracle ref)")]


def _rel(a, b):
    fin = np.isfinite(b)
    assert np.array_equal(fin, np.isfinite(a))
    return float((np.abs(a[fin] - b[fin]) / np.maximum(np.abs(b[fin]), 1.0)).max())


@pytest.mark.parametrize("which", ["tiny", "c1"])
def test_reference_pair_kernels_match_oracle(which, request):
    s = request.getfixturevalue(which)
    ds = s.dataset
    rp = mr.getparams(s.params15, ds.branchlengths)
    P, pi16, logw, *_ = mr.pair_categories(rp)
    ref_gpu = rk.pair_matrix(ds.children, ds.seqindex, ds.masks, P, pi16, logw, s.W)
    orc, _ = co.pair_matrix(ds.children, ds.seqindex, ds.masks, P, pi16, logw, s.W)
    assert _rel(ref_gpu, orc) < 1e-5
    from messi_gb300 import api
    from messi_gb300 import model as M
    ours, _ = api.felsensteincuda(ds, M.getparams(s.params15, ds.branchlengths), None, s.W)
    assert _rel(ours, ref_gpu) < 1e-5


def _scores(L, W, seed):
    rng = np.random.default_rng(seed)
    u = rng.uniform(-60.0, -20.0, L)
    p = np.full((L, L), -np.inf)
    for i in range(L):
        j = np.arange(i + 1, min(L, i + W + 1))
        p[i, j] = u[i] + u[j] + rng.normal(-3.0, 4.0, len(j))
    return u, np.maximum(p, p.T)


@pytest.mark.parametrize("L,W", [(17, 16), (64, 20), (150, 149)])
def test_reference_inside_outside_kernels_match_oracle(L, W):
    u, p = _scores(L, W, L + W)
    ins = co.inside(u, p)
    Zref = ins[0, 0, L - 1]
    Zk, tab = rk.inside(u, p)
    assert abs(Zk - Zref) <= 1e-5 * abs(Zref)
    tab = np.where(tab <= -1e19, -np.inf, tab)
    i, j = np.meshgrid(np.arange(L), np.arange(L), indexing="ij")
    band = (j >= i) & (j - i <= W)
    for X in range(3):
        r, g = ins[X][band], tab[X][band]
        fin = np.isfinite(r) & (r > -1e19)
        assert np.all(np.abs(g[fin] - r[fin]) <= 1e-5 * np.abs(r[fin]) + 1e-2)
    outs = co.outside(ins, u, p)
    otab = rk.outside(ins, u, p)
    otab = np.where(otab <= -1e19, -np.inf, otab)
    for X in range(3):
        r, g = outs[X][band], otab[X][band]
        fin = np.isfinite(r)
        assert np.all(np.abs(g[fin] - r[fin]) <= 1e-5 * np.abs(r[fin]) + 1e-2)
    from messi_gb300 import api
    assert abs(api.computeinsideKH99(u, p) - Zk) <= 1e-5 * abs(Zk)
