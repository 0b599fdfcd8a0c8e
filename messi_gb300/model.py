"""Model parameters, mirroring MESSI's parameter handling.

Host-side mirror of src/FARCE.jl:461-503 (``ModelParameters``),
:583-607 (``getparamsvector``), :609-657 (``getparams``), :699-740
(``MuseSpecificParameters`` / ``getmusespecificparamsarray``),
:1531-1583 (``discretizegamma`` / ``discretizegamma3``) and
:2398-2436 (``computeprior``).  The GPU library receives the discretised
categories (``ModelParameters.to_c``); the 16x16 rate matrices and their
exponentials are built inside the library.

``gtr``/``musefreqs``/``muse`` (src/RateMatrices.jl) are also provided in numpy
for the synthetic-data simulator.
"""
import math
from dataclasses import dataclass, field
from typing import List

import numpy as np
from scipy.stats import beta as _beta
from scipy.stats import gamma as _gamma

# src/MESSI.jl:1479-1480 (default starting vector, entry 10 reset to 1.0)
DEFAULT_PARAMS15 = np.array([2.0, 2.0, 2.0, 1.7487740904105369, 4.464074402974858, 1.6941505179847807,
                             0.4833108030758708, 5.839004646491171, 0.7168678100059017, 1.0, 0.6118067582467858,
                             0.23307618715645315, 0.2631203272837885, 0.2430685428508905, 0.5])

BASEPAIRINGS = (0, 0, 0, 2, 0, 0, 1, 0, 0, 1, 0, 3, 2, 0, 3, 0)


def discretizegamma(shape, scale, numcategories):
    """Gamma quantiles at the category mid-points (src/FARCE.jl:1531-1540)."""
    if numcategories == 1:
        return np.array([1.0])
    if numcategories == 0:  # Julia's empty comprehension (lambdaCats = 1)
        return np.zeros(0)
    w = 1.0 / numcategories
    return _gamma.ppf(np.array([w / 2.0 + i * w for i in range(numcategories)]), shape, scale=scale)


def discretizegamma3(lambdazeroweight, meanGC, meanAT, meanGT, gammavar, numcategories):
    """Lambda categories: rate 0 plus Gamma quantiles (src/FARCE.jl:1566-1583)."""
    rates = np.concatenate([[0.0], discretizegamma(gammavar, 1.0 / gammavar, numcategories)])
    # with no Gamma categories only the rate-0 category remains, weighted w0
    weights = np.ones(numcategories + 1) / max(numcategories, 1) * (1.0 - lambdazeroweight)
    weights[0] = lambdazeroweight
    return (weights, rates * (meanGC - 1.0), weights.copy(), rates * (meanAT - 1.0), weights.copy(),
            rates * (meanGT - 1.0))


@dataclass
class MuseSpecificParameters:
    """src/FARCE.jl:699-712."""
    lambdacat: int
    prob: float
    lambdarate: float
    lambdaGC: float
    lambdaAT: float
    lambdaGT: float

    @property
    def logprob(self):
        return math.log(self.prob) if self.prob > 0 else -math.inf


@dataclass
class ModelParameters:
    """src/FARCE.jl:461-503 (fields used by the likelihood path)."""
    freqs: np.ndarray
    lambdaGC: float
    lambdaAT: float
    lambdaGT: float
    q1: float
    q2: float
    q3: float
    q4: float
    q5: float
    q6: float
    branchlengths: np.ndarray
    lambdazeroweight: float = 0.5
    lambdaratesGC: np.ndarray = field(default_factory=lambda: np.ones(1))
    lambdaweightsGC: np.ndarray = field(default_factory=lambda: np.ones(1))
    lambdaratesAT: np.ndarray = field(default_factory=lambda: np.ones(1))
    lambdaweightsAT: np.ndarray = field(default_factory=lambda: np.ones(1))
    lambdaratesGT: np.ndarray = field(default_factory=lambda: np.ones(1))
    lambdaweightsGT: np.ndarray = field(default_factory=lambda: np.ones(1))
    lambdaCats: int = 1
    lambdaGammaShapeGC: float = 1.0
    lambdaGammaScaleGC: float = 1.0
    lambdaGammaShapeAT: float = 1.0
    lambdaGammaScaleAT: float = 1.0
    lambdaGammaShapeGT: float = 1.0
    lambdaGammaScaleGT: float = 1.0
    siteRates: np.ndarray = field(default_factory=lambda: np.ones(1))
    siteWeights: np.ndarray = field(default_factory=lambda: np.ones(1))
    siteCats: int = 1
    siteGammaShape: float = 1.0
    siteGammaScale: float = 1.0
    logposterior: float = 0.0
    loglikelihood: float = 0.0
    logprior: float = 0.0

    @property
    def q(self):
        return np.array([self.q1, self.q2, self.q3, self.q4, self.q5, self.q6])


def getparams(params, dataset, siteCats=3, lambdaCats=5, parameterisation=1, fixGU=False, fixGCAU=False):
    """15-vector -> ModelParameters (src/FARCE.jl:609-657).

    ``dataset`` may be a Dataset or an array of per-node branch lengths."""
    p = np.asarray(params, dtype=np.float64)
    if p.shape != (15,):
        raise ValueError("getparams expects the 15-entry parameter vector")
    bl = np.asarray(getattr(dataset, "branchlengths", dataset), dtype=np.float64)
    freqs = np.array([p[11], p[12], p[13], 1.0 - p[11] - p[12] - p[13]])
    cp = ModelParameters(freqs=freqs, lambdaGC=p[0], lambdaAT=p[1], lambdaGT=p[2], q1=p[3], q2=p[4], q3=p[5],
                         q4=p[6], q5=p[7], q6=p[8], branchlengths=bl.copy(), lambdazeroweight=p[14])
    cp.lambdaGammaShapeGC = p[9]
    cp.siteGammaShape = p[10]
    cp.siteGammaScale = 1.0 / cp.siteGammaShape
    cp.lambdaCats = lambdaCats - 1
    (cp.lambdaweightsGC, cp.lambdaratesGC, cp.lambdaweightsAT, cp.lambdaratesAT, cp.lambdaweightsGT,
     cp.lambdaratesGT) = discretizegamma3(cp.lambdazeroweight, cp.lambdaGC, cp.lambdaAT, cp.lambdaGT,
                                          cp.lambdaGammaScaleGC, cp.lambdaCats)
    if fixGCAU:
        cp.lambdaratesGC = cp.lambdaratesAT.copy()
    if fixGU:
        cp.lambdaratesGT = np.zeros(len(cp.lambdaratesGT))
    cp.siteCats = siteCats
    cp.siteWeights = np.ones(siteCats) / siteCats
    cp.siteRates = discretizegamma(cp.siteGammaShape, cp.siteGammaScale, siteCats)
    if len(cp.lambdaweightsGC) == 1:
        cp.lambdaratesGC = np.array([cp.lambdaGC - 1.0])
        cp.lambdaratesAT = np.array([cp.lambdaAT - 1.0])
        cp.lambdaratesGT = np.array([cp.lambdaGT - 1.0])
        cp.lambdaweightsGC = cp.lambdaweightsAT = cp.lambdaweightsGT = np.array([1.0])
    return cp


def getparamsvector(params):
    """ModelParameters -> 15-vector (src/FARCE.jl:583-607)."""
    return np.array([params.lambdaGC, params.lambdaAT, params.lambdaGT, params.q1, params.q2, params.q3, params.q4,
                     params.q5, params.q6, params.lambdaGammaShapeGC, params.siteGammaShape, params.freqs[0],
                     params.freqs[1], params.freqs[2], params.lambdazeroweight])


def getmusespecificparamsarray(params) -> List[MuseSpecificParameters]:
    """src/FARCE.jl:714-727."""
    out = []
    for k, (w, r) in enumerate(zip(params.lambdaweightsGC, params.lambdaratesGC)):
        out.append(MuseSpecificParameters(k + 1, float(w), float(r), params.lambdaGC, params.lambdaAT,
                                          params.lambdaGT))
    return out


def computeprior(params, samplebranchlengths=False, fixLambdaGT=False):
    """src/FARCE.jl:2398-2436."""
    pr = -(params.lambdaGC - 1.0) * 0.1 - (params.lambdaAT - 1.0) * 0.1
    if not fixLambdaGT:
        pr += -(params.lambdaGT - 1.0) * 0.1
    pr += -0.1 * (params.q1 + params.q2 + params.q3 + params.q4 + params.q5 + params.q6)
    if samplebranchlengths:
        pr += -0.2 * float(np.sum(params.branchlengths[1:]))
    pr += -0.1 * (params.lambdaGammaShapeGC + params.lambdaGammaScaleGC + params.lambdaGammaShapeAT +
                  params.lambdaGammaScaleAT + params.lambdaGammaShapeGT + params.lambdaGammaScaleGT)
    pr += -0.1 * params.siteGammaShape
    pr += float(_beta.logpdf(params.lambdazeroweight, 2.0, 2.0))
    return pr


# --------------------------------------------------------------------------
# numpy rate matrices (src/RateMatrices.jl), used by the simulator
# --------------------------------------------------------------------------
def gtr(q, piv):
    S = np.zeros((4, 4))
    for k, (i, j) in enumerate([(0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3)]):
        S[i, j] = S[j, i] = q[k]
    S = S * np.asarray(piv, dtype=np.float64)[None, :]
    return S - np.diag(S.sum(axis=1))


def musefreqs(pi4, lGC, lAT, lGT):
    lam = (1.0, lGC, lAT, lGT)
    f = np.outer(pi4, pi4).ravel() * np.array([lam[c] ** 2 for c in BASEPAIRINGS])
    return f / f.sum()


def muse(lGC, lAT, lGT, q, pi4, sr1=1.0, sr2=1.0):
    lam = (1.0, lGC, lAT, lGT)
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
            Q[h, v] = g[frm, to] * sr * pi4[to] * lam[BASEPAIRINGS[v]] / lam[BASEPAIRINGS[h]]
    return Q - np.diag(Q.sum(axis=1))
