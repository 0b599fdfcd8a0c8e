"""Golden outputs of the reference's own CUDA kernels, for the CPU test suite.

src/cuda/felsenstein.cu and src/cuda/inside.cu, compiled unmodified for
sm_103a (``make -C oracle ref``), run through oracle/ref_kernels.py (the
reference's launch sequences) on seeded synthetic inputs.  The inputs are
stored with the outputs, so tests/test_reference_fixtures.py checks the FP64
oracle against them on a machine without a GPU.  Needs a GPU and the
reference cubins:

    python tests/golden/make_reference_fixtures.py [out.npz]
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from messi_gb300 import synth  # noqa: E402
from oracle import c_oracle as co  # noqa: E402
from oracle import model_ref as mr  # noqa: E402
from oracle import ref_kernels as rk  # noqa: E402

WORKLOADS = {
    "tiny": (dict(numseqs=6, numcols=14, W=13, paired=0.3, mean_bl=0.15), 7),
    "c1": ("c1", 1),
}
INSIDE_CASES = [(17, 16), (40, 12)]
DECODING_CASES = [9, 30]


def inside_scores(L, W, seed):
    rng = np.random.default_rng(seed)
    u = rng.uniform(-60.0, -20.0, L)
    p = np.full((L, L), -np.inf)
    for i in range(L):
        j = np.arange(i + 1, min(L, i + W + 1))
        p[i, j] = u[i] + u[j] + rng.normal(-3.0, 4.0, len(j))
    return u, np.maximum(p, p.T)


def decoding_inputs(L, seed):
    rng = np.random.default_rng(seed)
    u = rng.uniform(-30.0, -8.0, L)
    p = np.full((L, L), -np.inf)
    for i in range(L):
        for j in range(i + 1, L):
            odds = rng.normal(-2.0, 3.0) + (rng.random() < 0.08) * rng.uniform(6, 18)
            p[i, j] = p[j, i] = u[i] + u[j] + odds
    ins = co.inside(u, p)
    outs = co.outside(ins, u, p)
    return co.basepairprobs(ins, outs, u, p)


def main(out):
    if not rk.available():
        raise SystemExit("reference cubins not built (make -C oracle ref)")
    f = {}
    for name, (spec, seed) in WORKLOADS.items():
        s = synth.make_workload(spec, seed=seed)
        ds = s.dataset
        rp = mr.getparams(s.params15, ds.branchlengths)
        P, pi16, logw, *_ = mr.pair_categories(rp)
        f[f"pairs_{name}_children"] = np.asarray(ds.children, np.int64)
        f[f"pairs_{name}_seqindex"] = np.asarray(ds.seqindex, np.int64)
        f[f"pairs_{name}_masks"] = np.asarray(ds.masks, np.uint8)
        f[f"pairs_{name}_params15"] = np.asarray(s.params15, np.float64)
        f[f"pairs_{name}_branchlengths"] = np.asarray(ds.branchlengths, np.float64)
        f[f"pairs_{name}_W"] = np.int64(s.W)
        f[f"pairs_{name}_ref"] = rk.pair_matrix(ds.children, ds.seqindex, ds.masks, P, pi16, logw, s.W)
    for L, W in INSIDE_CASES:
        u, p = inside_scores(L, W, L + W)
        Z, tab = rk.inside(u, p)
        f[f"inside_{L}_u"], f[f"inside_{L}_p"] = u, p
        f[f"inside_{L}_Z"] = np.float64(Z)
        f[f"inside_{L}_tab"] = tab
        f[f"inside_{L}_W"] = np.int64(W)
        f[f"outside_{L}_tab"] = rk.outside(co.inside(u, p), u, p)
    for L in DECODING_CASES:
        single, pair = decoding_inputs(L, 3 * L)
        e, sm = rk.posterior_decoding(single, pair, 2.0)
        f[f"decoding_{L}_single"], f[f"decoding_{L}_pair"] = single, pair
        f[f"decoding_{L}_e"], f[f"decoding_{L}_s"] = e, sm
    np.savez_compressed(out, **f)
    print(f"wrote {out}: {len(f)} arrays, {os.path.getsize(out)} bytes")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.path.join(os.path.dirname(os.path.abspath(__file__)),
                                                            "reference_outputs.npz"))
