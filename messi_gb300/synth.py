"""Seeded synthetic alignments with the shapes of MESSI's benchmark workloads.

Generative recipe after src/Simulations.jl:72-184 (``simulatealignments``):
a random nested structure, unpaired columns drawn from the GTR x site-rate
model and paired columns from the 16-state paired model of a category drawn
by its weight, each sampled down the tree from the root frequencies
(``backwardssampling``, src/Simulations.jl:47-70, with flat likelihoods).
The paired digit order follows the likelihood's convention (first digit =
left column, src/cuda/felsenstein.cu:129).

Named workloads (seeded ``numpy.random.Generator(PCG64(seed))``):
  "c1": 16 seqs x 120 nt, every pair (W = 119), 30% paired, mean branch 0.1
  "c2": 64 seqs x 1,000 nt, max pair span 500, 30% paired, mean branch 0.1
  "c4": 30 seqs x 9,000 nt, max pair span 800, 20% paired, mean branch 0.05
  "c2p": 64 seqs x 600 nt, max pair span 300 (profiling-sized c2)
Batches (``make_batch``): "c3" = 256 alignments, each with L ~ U(80, 1500)
columns, N ~ U(8, 128) sequences, W = L - 1, its own tree, structure and
model; "c3s" = 24 alignments, L ~ U(20, 160), N ~ U(4, 24) (test-sized).
Every workload: pi ~ Dirichlet(5,5,5,5), lambda_GC/AT/GT ~ U(1,5), exchange
rates and site-rate shape at the reference's starting vector
(src/MESSI.jl:1479), 5% i.i.d. gaps.
"""
from dataclasses import dataclass

import numpy as np

from . import model as M
from .dataset import Dataset, TreeNode, to_newick

WORKLOADS = {
    "c1": dict(numseqs=16, numcols=120, W=119, paired=0.30, mean_bl=0.10),
    "c2": dict(numseqs=64, numcols=1000, W=500, paired=0.30, mean_bl=0.10),
    "c4": dict(numseqs=30, numcols=9000, W=800, paired=0.20, mean_bl=0.05),
    # profiling-sized case of the c2 shape (about 2 GB of partials)
    "c2p": dict(numseqs=64, numcols=600, W=300, paired=0.30, mean_bl=0.10),
    # profiling-sized case with the c4 band (the same inside/outside passes,
    # 8 sequences so that the pair pruning holds little memory)
    "c4p": dict(numseqs=8, numcols=9000, W=800, paired=0.20, mean_bl=0.05),
}


@dataclass
class Synthetic:
    dataset: Dataset
    params15: np.ndarray
    paired: np.ndarray   # partner column or -1
    W: int
    fasta: str
    newick: str
    seed: int


def random_unrooted_tree(rng, n, mean_bl):
    """Random unrooted binary topology by sequential leaf insertion on a random
    edge, with a trifurcating root (as FastTree writes) and Exp(mean_bl)
    branch lengths."""
    if n < 3:
        raise ValueError("need at least 3 sequences")
    root = TreeNode(0.0, "")
    leaves = []
    for k in range(3):
        leaf = TreeNode(0.0, f"seq{k + 1}")
        root.addchild(leaf)
        leaves.append(leaf)
    nodes = list(leaves)
    for k in range(3, n):
        v = nodes[rng.integers(0, len(nodes))]
        par = v.parent
        w = TreeNode(0.0, "")
        idx = par.children.index(v)
        par.children[idx] = w
        w.parent = par
        v.parent = None
        w.addchild(v)
        leaf = TreeNode(0.0, f"seq{k + 1}")
        w.addchild(leaf)
        nodes.extend([w, leaf])
    for v in nodes:
        v.branchlength = float(rng.exponential(mean_bl))
    return root


def random_structure(rng, L, W, frac, minloop=3, maxhelix=8):
    """Random nested structure pairing about `frac` of the columns, every pair
    spanning at most W columns and enclosing at least `minloop` - 1 columns."""
    paired = -np.ones(L, dtype=np.int64)
    target = int(round(frac * L))
    npaired = 0
    attempts = 0
    maxspan = min(W, L - 1)
    if maxspan < minloop:
        return paired
    while npaired + 2 <= target and attempts < 50 * L:
        attempts += 1
        i = int(rng.integers(0, L - minloop))
        span = int(rng.integers(minloop, maxspan + 1))
        j = i + span
        if j >= L:
            continue
        h = int(rng.integers(3, maxhelix + 1))
        added = 0
        for k in range(h):
            a, b = i + k, j - k
            if b - a < minloop or paired[a] >= 0 or paired[b] >= 0:
                break
            inner = paired[a + 1:b]
            sel = inner >= 0
            if sel.any():
                part = inner[sel]
                if (part <= a).any() or (part >= b).any():
                    break
            paired[a], paired[b] = b, a
            added += 2
            if npaired + added + 2 > target:
                break
        npaired += added
    return paired


def _sample_rows(rng, rows):
    cum = np.cumsum(rows, axis=1)
    u = rng.random(rows.shape[0]) * cum[:, -1]
    return np.minimum((u[:, None] > cum).sum(axis=1), rows.shape[1] - 1)


def _simulate_down(rng, ds, Pn, rootprob, ncols):
    """Sample states down the tree for `ncols` columns; Pn[v] is an array
    (ncols, n, n) of per-column transition matrices for node v."""
    states = np.zeros((ds.numnodes, ncols), dtype=np.int64)
    states[0] = _sample_rows(rng, rootprob)
    for v in range(1, ds.numnodes):
        p = ds.parent[v]
        rows = Pn[v][np.arange(ncols), states[p]]
        states[v] = _sample_rows(rng, rows)
    return states


def _pmats(Q, pi, bls):
    """exp(Q t) for every branch length (reversible Q with stationary pi, by
    the symmetric eigendecomposition); zero matrix for the root (index 0)."""
    d = np.sqrt(pi)
    S = (d[:, None] * Q) / d[None, :]
    w, U = np.linalg.eigh(0.5 * (S + S.T))
    t = np.asarray(bls, np.float64)
    E = np.exp(w[None, :] * t[:, None])
    P = np.einsum("ak,nk,dk->nad", U, E, U) * (d[None, None, :] / d[None, :, None])
    P = np.maximum(P, 0.0)
    P[0] = 0.0
    return P


def simulate(rng, ds, params15, paired, gap_rate=0.05):
    """Fill the alignment of `ds` (its tree only is used) from the model."""
    cp = M.getparams(params15, ds.branchlengths, 3, 5)
    L = ds.numcols
    N = ds.numseqs
    nodes = ds.numnodes
    # unpaired model: GTR x site rate (src/Simulations.jl:99-107)
    Q4 = M.gtr(cp.q, cp.freqs)
    P4 = np.array([_pmats(Q4 * r, cp.freqs, ds.branchlengths) for r in cp.siteRates])
    # paired model: 45 categories with weights (src/Simulations.jl:110-128)
    museparams = M.getmusespecificparamsarray(cp)
    cats, logw = [], []
    for a in range(3):
        for b in range(3):
            for mp in museparams:
                cats.append((a, b, mp))
                logw.append(np.log(cp.siteWeights[a]) + np.log(cp.siteWeights[b]) + mp.logprob)
    logw = np.array(logw)
    catprob = np.exp(logw - logw.max())
    catprob /= catprob.sum()
    seqs = np.zeros((N, L), dtype=np.int64)
    unp = np.where(paired < 0)[0]
    if len(unp):
        z = rng.choice(len(cp.siteRates), size=len(unp), p=cp.siteWeights)
        Pn = [P4[z, v] for v in range(nodes)]
        st = _simulate_down(rng, ds, Pn, np.tile(cp.freqs, (len(unp), 1)), len(unp))
        for v in range(nodes):
            if ds.seqindex[v] >= 0:
                seqs[ds.seqindex[v], unp] = st[v]
    left = np.where(paired > np.arange(L))[0]
    if len(left):
        z = rng.choice(len(cats), size=len(left), p=catprob)
        used = np.unique(z)
        P16 = {}
        pi16 = {}
        for c in used:
            a, b, mp = cats[c]
            lGC, lAT, lGT = cp.lambdaratesGC[mp.lambdacat - 1] + 1, cp.lambdaratesAT[mp.lambdacat - 1] + 1, \
                cp.lambdaratesGT[mp.lambdacat - 1] + 1
            Q = M.muse(lGC, lAT, lGT, cp.q, cp.freqs, cp.siteRates[a], cp.siteRates[b])
            pi16[c] = M.musefreqs(cp.freqs, lGC, lAT, lGT)
            P16[c] = _pmats(Q, pi16[c], ds.branchlengths)
        idx = {c: k for k, c in enumerate(used)}
        stack = np.array([P16[c] for c in used])       # [used, nodes, 16, 16]
        zi = np.array([idx[c] for c in z])
        Pn = [stack[zi, v] for v in range(nodes)]
        rootp = np.array([pi16[c] for c in z])
        st = _simulate_down(rng, ds, Pn, rootp, len(left))
        for v in range(nodes):
            if ds.seqindex[v] >= 0:
                seqs[ds.seqindex[v], left] = st[v] // 4
                seqs[ds.seqindex[v], paired[left]] = st[v] % 4
    letters = np.array(list("ACGU"))
    chars = letters[seqs]
    gaps = rng.random((N, L)) < gap_rate
    chars[gaps] = "-"
    return ["".join(row) for row in chars]


def make_workload(name_or_spec, seed=1):
    """Build one seeded synthetic workload (see module docstring)."""
    spec = dict(WORKLOADS[name_or_spec]) if isinstance(name_or_spec, str) else dict(name_or_spec)
    rng = np.random.Generator(np.random.PCG64(seed))
    N, L, W = spec["numseqs"], spec["numcols"], spec["W"]
    root = random_unrooted_tree(rng, N, spec["mean_bl"])
    newick = to_newick(root)
    names = [f"seq{k + 1}" for k in range(N)]
    ds = Dataset.from_sequences(names, ["A" * L] * N, newick)
    pi = rng.dirichlet([5.0, 5.0, 5.0, 5.0])
    lam = rng.uniform(1.0, 5.0, size=3)
    p15 = M.DEFAULT_PARAMS15.copy()
    p15[0:3] = lam
    p15[11:14] = pi[:3]
    paired = random_structure(rng, L, W, spec["paired"])
    seqs = simulate(rng, ds, p15, paired, spec.get("gap_rate", 0.05))
    fasta = "".join(f">{n}\n{s}\n" for n, s in zip(names, seqs))
    ds = Dataset.from_sequences(names, seqs, newick)
    return Synthetic(dataset=ds, params15=p15, paired=paired, W=W, fasta=fasta, newick=newick, seed=seed)


BATCHES = {
    "c3": dict(count=256, numcols=(80, 1500), numseqs=(8, 128), paired=0.30, mean_bl=0.10),
    "c3s": dict(count=24, numcols=(20, 160), numseqs=(4, 24), paired=0.30, mean_bl=0.10),
}


def make_batch(name, seed=1):
    """Seeded batch of independent workloads (see module docstring); the
    band of each alignment is its full length (W = L - 1)."""
    spec = BATCHES[name]
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for k in range(spec["count"]):
        L = int(rng.integers(spec["numcols"][0], spec["numcols"][1] + 1))
        N = int(rng.integers(spec["numseqs"][0], spec["numseqs"][1] + 1))
        one = dict(numseqs=max(3, N), numcols=L, W=max(1, L - 1), paired=spec["paired"], mean_bl=spec["mean_bl"])
        out.append(make_workload(one, seed=int(rng.integers(1, 2 ** 31))))
    return out
