"""Independent numpy / pure-Python restatement for tiny cases.

TEST INFRASTRUCTURE ONLY (see oracle/__init__.py).  It shares no code with
messi_oracle.c: P = exp(Qt) comes from scipy.linalg.expm, pruning runs
without pattern caching or rescaling, and the SCFG recurrences are written
from the grammar (src/InsideOutsideAlgorithm.jl:30-53) as plain loops.  It is
used to cross-check the C oracle and to enumerate structures for the
brute-force known-answer test.
"""
import itertools

import numpy as np
from scipy.linalg import expm

R = np.log(np.array([0.868534, 0.117609877998, 0.013856122002, 0.787640, 0.21236, 0.894603, 0.105397]))
BASEPAIRINGS = [0, 0, 0, 2, 0, 0, 1, 0, 0, 1, 0, 3, 2, 0, 3, 0]


def gtr(q, piv):
    S = np.zeros((4, 4))
    idx = [(0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3)]
    for k, (i, j) in enumerate(idx):
        S[i, j] = S[j, i] = q[k]
    S = S * np.asarray(piv)[None, :]
    return S - np.diag(S.sum(axis=1))


def musefreqs(pi, lGC, lAT, lGT):
    lam = [1.0, lGC, lAT, lGT]
    f = np.outer(pi, pi).ravel() * np.array([lam[c] ** 2 for c in BASEPAIRINGS])
    return f / f.sum()


def muse(lGC, lAT, lGT, q, pi, sr1, sr2):
    lam = [1.0, lGC, lAT, lGT]
    g = gtr(q, np.ones(4))
    Q = np.zeros((16, 16))
    for h in range(16):
        for v in range(16):
            if h == v:
                continue
            if h // 4 == v // 4:
                frm, to, sr = h % 4, v % 4, sr2
            elif h % 4 == v % 4:
                frm, to, sr = h // 4, v // 4, sr1
            else:
                continue
            Q[h, v] = g[frm, to] * sr * pi[to] * lam[BASEPAIRINGS[v]] / lam[BASEPAIRINGS[h]]
    return Q - np.diag(Q.sum(axis=1))


def transition_matrices(Q, branchlengths):
    n = Q.shape[0]
    P = [np.zeros((n, n))]
    for t in branchlengths[1:]:
        M = expm(Q * t)
        M[M <= 0] = 1e-50
        P.append(M)
    return np.array(P)


def leafvec(mask):
    return np.array([(mask >> a) & 1 for a in range(4)], dtype=np.float64)


def prune_column_pair(children, seqindex, masks, P, pi, x, y=None):
    """log P(columns | tree) by plain recursion (tiny trees only)."""

    def rec(v):
        c0, c1 = children[v]
        if c0 < 0:
            s = seqindex[v]
            a = leafvec(masks[s, x])
            return a if y is None else np.kron(a, leafvec(masks[s, y]))
        return (P[c0] @ rec(c0)) * (P[c1] @ rec(c1))

    return float(np.log(pi @ rec(0)))


def inside(u, p):
    L = len(u)
    I = np.full((3, L, L), -np.inf)
    for i in range(L):
        I[0, i, i] = u[i] + R[1]
        I[2, i, i] = u[i] + R[5]
    for d in range(1, L):
        for i in range(L - d):
            j = i + d
            tmp = -np.inf
            for h in range(i, j):
                tmp = np.logaddexp(tmp, I[2, i, h] + I[0, h + 1, j])
            fin = I[1, i + 1, j - 1] if d >= 2 else -np.inf
            v = p[i, j] + fin
            I[0, i, j] = np.logaddexp(R[0] + tmp, R[2] + v)
            I[1, i, j] = np.logaddexp(R[4] + tmp, R[3] + v)
            I[2, i, j] = R[6] + v
    return I


def _structures(i, j, minloop=3):
    """All nested pair sets on [i, j] whose pairs span at least `minloop`."""
    if j < i:
        yield ()
        return
    # i unpaired
    for s in _structures(i + 1, j, minloop):
        yield s
    # i paired with k
    for k in range(i + minloop, j + 1):
        for a in _structures(i + 1, k - 1, minloop):
            for b in _structures(k + 1, j, minloop):
                yield ((i, k),) + a + b


def kh99_prior(paired, L):
    """log prior of a structure under KH99 (src/InsideOutsideAlgorithm.jl:86-144)."""
    # unfolded rules: S->sS, S->dFdS, S->s, S->dFd, F->dFd, F->sS, F->dFdS, L->s, L->dFd
    rules = {
        ("S", "sS"): R[0] + R[5], ("S", "dFdS"): R[0] + R[6], ("S", "s"): R[1], ("S", "dFd"): R[2],
        ("F", "dFd"): R[3], ("F", "sS"): R[4] + R[5], ("F", "dFdS"): R[4] + R[6],
    }
    ll = 0.0
    stack = [("S", 0, L - 1)]
    while stack:
        sym, s, e = stack.pop()
        if paired[s] < 0:
            if s == e:
                ll += rules[(sym, "s")] if (sym, "s") in rules else -np.inf
            else:
                ll += rules[(sym, "sS")]
                stack.append(("S", s + 1, e))
        else:
            k = paired[s]
            if k == e:
                ll += rules[(sym, "dFd")]
                stack.append(("F", s + 1, k - 1))
            else:
                ll += rules[(sym, "dFdS")]
                stack.append(("F", s + 1, k - 1))
                stack.append(("S", k + 1, e))
    return ll


def brute_force_Z(u, p):
    """log sum over all structures of prior x emissions (L <= ~10)."""
    L = len(u)
    Z = -np.inf
    for pairs in _structures(0, L - 1):
        paired = -np.ones(L, dtype=int)
        for (a, b) in pairs:
            paired[a], paired[b] = b, a
        ll = kh99_prior(paired, L)
        for x in range(L):
            if paired[x] < 0:
                ll += u[x]
            elif paired[x] > x:
                ll += p[x, paired[x]]
        Z = np.logaddexp(Z, ll)
    return Z


def brute_force_posteriors(u, p):
    """Posterior pairing probabilities by enumeration (row-normalised like
    src/InsideOutsideAlgorithm.jl:518-527)."""
    L = len(u)
    single = np.zeros(L)
    pair = np.zeros((L, L))
    lls, structs = [], []
    for pairs in _structures(0, L - 1):
        paired = -np.ones(L, dtype=int)
        for (a, b) in pairs:
            paired[a], paired[b] = b, a
        ll = kh99_prior(paired, L)
        for x in range(L):
            if paired[x] < 0:
                ll += u[x]
            elif paired[x] > x:
                ll += p[x, paired[x]]
        lls.append(ll)
        structs.append(paired)
    lls = np.array(lls)
    w = np.exp(lls - lls.max())
    w /= w.sum()
    for wi, paired in zip(w, structs):
        for x in range(L):
            if paired[x] < 0:
                single[x] += wi
            else:
                pair[x, paired[x]] += wi
    s = single + pair.sum(axis=1)
    return single / s, pair / s[:, None]


def decoding_score(pairs, single, pair, alpha, i, j):
    """Objective of the posterior-decoding recursion (src/cuda/inside.cu:286-321)
    for one nested structure on [i, j]: the segment decomposition the
    recursion uses (first column unpaired / paired with the segment end /
    paired inside), with e(i, i) = 0."""
    if j <= i:
        return 0.0
    partner = dict(pairs)
    partner.update({b: a for a, b in pairs})
    k = partner.get(i)
    if k is None or k < i:
        return single[i] + decoding_score(pairs, single, pair, alpha, i + 1, j)
    if k == j:
        return alpha * pair[i][j] + decoding_score(pairs, single, pair, alpha, i + 1, j - 1)
    return (alpha * pair[i][k] + decoding_score(pairs, single, pair, alpha, i + 1, k - 1)
            + decoding_score(pairs, single, pair, alpha, k + 1, j))


def brute_force_decoding(single, pair, alpha):
    """(best score, best pair set) over every nested structure on L columns
    (adjacent pairs allowed, as in the decoding recursion)."""
    L = len(single)
    best, arg = -np.inf, None
    for s in _structures(0, L - 1, minloop=1):
        v = decoding_score(s, single, pair, alpha, 0, L - 1)
        if v > best:
            best, arg = v, s
    return best, arg
