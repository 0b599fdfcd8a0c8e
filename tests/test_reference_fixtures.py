"""The FP64 oracle against golden outputs of the reference's own CUDA
kernels (src/cuda/felsenstein.cu, src/cuda/inside.cu compiled unmodified and
run with the reference's launch sequences on seeded synthetic inputs; the
arrays and the script that wrote them are in tests/golden/).  The reference
kernels compute in FP32, so the tolerances are FP32-sized, as in
tests/test_gpu_reference_kernels.py; posterior decoding is bit-exact.  No
GPU needed."""
import os

import numpy as np
import pytest

from oracle import c_oracle as co
from oracle import model_ref as mr

PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_outputs.npz")


@pytest.fixture(scope="module")
def gold():
    return np.load(PATH)


def _rel(a, b):
    fin = np.isfinite(b)
    assert np.array_equal(fin, np.isfinite(a))
    return float((np.abs(a[fin] - b[fin]) / np.maximum(np.abs(b[fin]), 1.0)).max())


@pytest.mark.parametrize("name", ["tiny", "c1"])
def test_oracle_pair_matrix_matches_reference_kernels(gold, name):
    def g(k):
        return gold[f"pairs_{name}_{k}"]

    rp = mr.getparams(g("params15"), g("branchlengths"))
    P, pi16, logw, *_ = mr.pair_categories(rp)
    orc, _ = co.pair_matrix(g("children"), g("seqindex"), g("masks"), P, pi16, logw, int(g("W")))
    assert _rel(g("ref"), orc) < 1e-5


@pytest.mark.parametrize("L", [17, 40])
def test_oracle_inside_outside_match_reference_kernels(gold, L):
    u, p, W = gold[f"inside_{L}_u"], gold[f"inside_{L}_p"], int(gold[f"inside_{L}_W"])
    ins = co.inside(u, p)
    Zref = ins[0, 0, L - 1]
    Zk = float(gold[f"inside_{L}_Z"])
    assert abs(Zk - Zref) <= 1e-5 * abs(Zref)
    i, j = np.meshgrid(np.arange(L), np.arange(L), indexing="ij")
    band = (j >= i) & (j - i <= W)
    tab = np.where(gold[f"inside_{L}_tab"] <= -1e19, -np.inf, gold[f"inside_{L}_tab"])
    for X in range(3):
        r, g = ins[X][band], tab[X][band]
        fin = np.isfinite(r) & (r > -1e19)
        assert np.all(np.abs(g[fin] - r[fin]) <= 1e-5 * np.abs(r[fin]) + 1e-2)
    outs = co.outside(ins, u, p)
    otab = np.where(gold[f"outside_{L}_tab"] <= -1e19, -np.inf, gold[f"outside_{L}_tab"])
    for X in range(3):
        r, g = outs[X][band], otab[X][band]
        fin = np.isfinite(r)
        assert np.all(np.abs(g[fin] - r[fin]) <= 1e-5 * np.abs(r[fin]) + 1e-2)


@pytest.mark.parametrize("L", [9, 30])
def test_oracle_posterior_decoding_matches_reference_kernel_bit_for_bit(gold, L):
    e, s = co.posterior_decoding(gold[f"decoding_{L}_single"], gold[f"decoding_{L}_pair"], 2.0)
    np.testing.assert_array_equal(e, gold[f"decoding_{L}_e"])
    np.testing.assert_array_equal(s, gold[f"decoding_{L}_s"])
