"""FP64 restatement of MESSI's parameter handling and likelihood entry point.

TEST INFRASTRUCTURE ONLY (see oracle/__init__.py).

* ``getparams``: src/FARCE.jl:609-657 (15-vector -> categories), with
  ``discretizegamma`` src/FARCE.jl:1531-1540 and ``discretizegamma3``
  src/FARCE.jl:1566-1583.  Distributions.jl's ``quantile(Gamma)`` is replaced
  by scipy's ``gamma.ppf`` (the reference's own Distributions 0.16.2 is not
  available here).
* ``pair_categories``: the (siteCat1, siteCat2, lambda) loop order of
  src/FelsensteinCUDA.jl:277-279 and src/FARCE.jl:1746-1755.
* ``computeprior``: src/FARCE.jl:2398-2436.
* ``structure_integrated_likelihood``: src/FARCE.jl:2322-2345 plus the
  ``maskgapped!`` call of src/MESSI.jl:310.
"""
from dataclasses import dataclass, field

import numpy as np
from scipy.stats import beta as _beta
from scipy.stats import gamma as _gamma

from . import c_oracle

# src/MESSI.jl:1479 (default starting vector; entry 10 is reset to 1.0 at :1480)
DEFAULT_PARAMS15 = np.array([2.0, 2.0, 2.0, 1.7487740904105369, 4.464074402974858, 1.6941505179847807,
                             0.4833108030758708, 5.839004646491171, 0.7168678100059017, 1.0, 0.6118067582467858,
                             0.23307618715645315, 0.2631203272837885, 0.2430685428508905, 0.5])


def discretizegamma(shape, scale, numcategories):
    if numcategories == 1:
        return np.array([1.0])
    if numcategories == 0:  # Julia's empty comprehension (lambdaCats = 1)
        return np.zeros(0)
    w = 1.0 / numcategories
    vs = np.array([w / 2.0 + i * w for i in range(numcategories)])
    return _gamma.ppf(vs, shape, scale=scale)


def discretizegamma3(lambdazeroweight, meanGC, meanAT, meanGT, gammavar, numcategories):
    rates = np.concatenate([[0.0], discretizegamma(gammavar, 1.0 / gammavar, numcategories)])
    # with no Gamma categories only the rate-0 category remains, weighted w0
    weights = np.ones(numcategories + 1) / max(numcategories, 1) * (1.0 - lambdazeroweight)
    weights[0] = lambdazeroweight
    return weights, rates * (meanGC - 1.0), rates * (meanAT - 1.0), rates * (meanGT - 1.0)


@dataclass
class RefParams:
    freqs: np.ndarray
    lambdaGC: float
    lambdaAT: float
    lambdaGT: float
    q: np.ndarray
    branchlengths: np.ndarray
    lambdazeroweight: float
    lambdaweights: np.ndarray
    lambdaratesGC: np.ndarray
    lambdaratesAT: np.ndarray
    lambdaratesGT: np.ndarray
    lambdaGammaShapeGC: float
    lambdaGammaScaleGC: float
    siteGammaShape: float
    siteRates: np.ndarray
    siteWeights: np.ndarray
    extra: dict = field(default_factory=dict)


def getparams(p15, branchlengths, siteCats=3, lambdaCats=5):
    p = np.asarray(p15, np.float64)
    freqs = np.array([p[11], p[12], p[13], 1.0 - p[11] - p[12] - p[13]])
    siteshape = p[10]
    weights, rGC, rAT, rGT = discretizegamma3(p[14], p[0], p[1], p[2], 1.0, lambdaCats - 1)
    if len(weights) == 1:
        rGC, rAT, rGT = np.array([p[0] - 1.0]), np.array([p[1] - 1.0]), np.array([p[2] - 1.0])
        weights = np.array([1.0])
    return RefParams(freqs=freqs, lambdaGC=p[0], lambdaAT=p[1], lambdaGT=p[2], q=p[3:9].copy(),
                     branchlengths=np.asarray(branchlengths, np.float64), lambdazeroweight=p[14],
                     lambdaweights=weights, lambdaratesGC=rGC, lambdaratesAT=rAT, lambdaratesGT=rGT,
                     lambdaGammaShapeGC=p[9], lambdaGammaScaleGC=1.0, siteGammaShape=siteshape,
                     siteRates=discretizegamma(siteshape, 1.0 / siteshape, siteCats),
                     siteWeights=np.ones(siteCats) / siteCats)


def pair_categories(rp):
    """(P, pi16, logw, lamidx, lambda1, site1, site2) for every category in the
    reference order: siteCat1 outer, siteCat2, lambda category inner."""
    Ps, pis, logw, lam, l1, s1, s2 = [], [], [], [], [], [], []
    nsite = len(rp.siteRates)
    for a in range(nsite):
        for b in range(nsite):
            for k in range(len(rp.lambdaweights)):
                lGC = rp.lambdaratesGC[k] + 1.0
                lAT = rp.lambdaratesAT[k] + 1.0
                lGT = rp.lambdaratesGT[k] + 1.0
                Q = c_oracle.muse(lGC, lAT, lGT, rp.q, rp.freqs, rp.siteRates[a], rp.siteRates[b])
                pi16 = c_oracle.musefreqs(rp.freqs, lGC, lAT, lGT)
                Ps.append(c_oracle.transition_matrices(Q, pi16, rp.branchlengths))
                pis.append(pi16)
                with np.errstate(divide="ignore"):
                    logw.append(np.log(rp.siteWeights[a]) + np.log(rp.siteWeights[b]) + np.log(rp.lambdaweights[k]))
                lam.append(k)
                l1.append(1 if (rp.lambdaratesGC[k] == 0.0 and rp.lambdaratesAT[k] == 0.0
                                and rp.lambdaratesGT[k] == 0.0) else 0)
                s1.append(a)
                s2.append(b)
    return (np.array(Ps), np.array(pis), np.array(logw), np.array(lam, np.int32), np.array(l1, np.int32),
            np.array(s1, np.int32), np.array(s2, np.int32))


def unpaired_categories(rp):
    """P4 per site-rate category (exp(Q*rate*t)), root freqs, log weights:
    src/FARCE.jl:742-750."""
    Q = c_oracle.gtr(rp.q, rp.freqs)
    P4 = np.array([c_oracle.transition_matrices(Q * r, rp.freqs, rp.branchlengths) for r in rp.siteRates])
    return P4, rp.freqs.copy(), np.log(rp.siteWeights)


def computeprior(rp):
    """src/FARCE.jl:2398-2436 (samplebranchlengths=false, fixLambdaGT=false)."""
    pr = -(rp.lambdaGC - 1.0) * 0.1 - (rp.lambdaAT - 1.0) * 0.1 - (rp.lambdaGT - 1.0) * 0.1
    pr += -0.1 * float(np.sum(rp.q))
    # lambdaGammaShape/Scale for GC, AT, GT: only the GC shape is a free
    # parameter; the other five keep their constructor default of 1.0
    pr += -0.1 * rp.lambdaGammaShapeGC - 0.1 * rp.lambdaGammaScaleGC - 0.1 * 4 * 1.0
    pr += -0.1 * rp.siteGammaShape
    pr += float(_beta.logpdf(rp.lambdazeroweight, 2.0, 2.0))
    return pr


def unpaired_loglik(tree, masks, rp):
    P4, pi4, logw = unpaired_categories(rp)
    return c_oracle.unpaired(tree["children"], tree["seqindex"], masks, P4, pi4, logw)


def pair_loglik(tree, masks, rp, W, pairmask=None, rows=None, nthreads=0, per_lambda=False,
                lambda1_factorised=False, u_by_site=None):
    P, pi16, logw, lam, l1, s1, s2 = pair_categories(rp)
    kw = {}
    if per_lambda:
        kw.update(lamidx=lam, nlam=len(rp.lambdaweights))
    if lambda1_factorised:
        kw.update(lambda1_cat=l1, u_by_site=u_by_site, site1=s1, site2=s2)
    return c_oracle.pair_matrix(tree["children"], tree["seqindex"], masks, P, pi16, logw, W, pairmask=pairmask,
                                rows=rows, nthreads=nthreads, **kw)


def structure_integrated_likelihood(tree, masks, gapfreq, p15, W, gapcutoff=1.0, nthreads=0, siteCats=3,
                                    lambdaCats=5):
    """logprior + Z: src/FARCE.jl:2322-2345, masked as at src/MESSI.jl:310."""
    rp = getparams(p15, tree["branchlengths"], siteCats, lambdaCats)
    u, _ = unpaired_loglik(tree, masks, rp)
    p, _ = pair_loglik(tree, masks, rp, W, nthreads=nthreads)
    p = c_oracle.maskgapped(p, gapfreq, gapcutoff)
    ins = c_oracle.inside(u, p, 1.0, nthreads=nthreads)
    Z = ins[0, 0, len(u) - 1]
    return computeprior(rp) + Z, dict(u=u, p=p, inside=ins, Z=Z, params=rp)


def siterate_conditionals(tree, masks, rp, W, single, pair, pairmask=None):
    """felsensteinposteriorsiterateconditionalscuda (src/FelsensteinCUDA.jl:
    518-717) in FP64: per site-rate category s and column x, the log-sum-exp
    of log w_s + log single[x] + u_s[x] and, over evaluated partners, of
    log pair + log w_c + ll_c for the categories whose rate at x is s
    (first column: siteCat1, second column: siteCat2)."""
    import numpy as np
    P, pi16, logw, lam, l1, s1, s2 = pair_categories(rp)
    C = P.shape[0]
    L = masks.shape[1]
    ns = len(rp.siteRates)
    _, ubs = unpaired_loglik(tree, masks, rp)
    out = np.full((ns, L), -np.inf)

    def lse(a, b):
        return np.logaddexp(a, b)
    for s in range(ns):
        for x in range(L):
            if np.isfinite(ubs[s, x]) and single[x] > 0:
                out[s, x] = np.log(rp.siteWeights[s]) + np.log(single[x]) + ubs[s, x]
    for c in range(C):
        llc, _ = c_oracle.pair_matrix(tree["children"], tree["seqindex"], masks, P[c:c + 1], pi16[c:c + 1],
                                      np.zeros(1), W, pairmask=pairmask)
        for x in range(L):
            for y in range(x + 1, min(L, x + W + 1)):
                if not np.isfinite(llc[x, y]) or not (pair[x, y] > 0):
                    continue
                v = np.log(pair[x, y]) + logw[c] + llc[x, y]
                out[s1[c], x] = lse(out[s1[c], x], v)
                out[s2[c], y] = lse(out[s2[c], y], v)
    return out
