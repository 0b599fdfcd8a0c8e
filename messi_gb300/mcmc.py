"""MCMC over the model parameters with the GPU likelihood (HP3).

The reference's chain (src/MCMC.jl:675-1868, ``runchain``) samples the
parameters of the structure-integrated likelihood; its default move mixture
(src/default.params, ``moveweights``) is dominated by move 8, the adaptive
random walk of ``gettunedparams`` (src/MCMC.jl:393-449) over the 14-entry
tuning vector (``gettuningvector``/``settuningparams``, :307-370), accepted by
Metropolis-Hastings (:1666).  This module provides:

* the target: ``computeprior`` + Z from ``messi_likelihood`` (all on the GPU);
* ``PlainProposal``: move 8 restated (its five masked sub-moves and the
  isotropic-then-adaptive covariance);
* ``LearnedProposal``: a K-component Gaussian mixture in an unconstrained
  parameter space whose weights/means/scales come from the BF16 MLP of
  ``api.MLP`` given the current state and alignment summaries.  It is trained
  on the chain's own states during burn-in and frozen afterwards; its density
  is evaluated in both directions, so the Metropolis-Hastings ratio is exact
  and the posterior is unchanged.  The plain move stays in the mixture of
  kernels as the fallback;
* ``ess`` (Geyer's initial monotone sequence) and ``mcse`` (batch means).

State.  After a move-8 step the reference's round trip ``settuningparams`` ->
``getparamsvector`` -> ``getparams`` ties the lambda gamma shape (p10) to
lambda_GC and resets the gamma scale, and move 8 never changes pi.  The chain
state is therefore the 11 free parameters (q1..q6, site-rate shape,
lambda-zero weight, lambda_GC, lambda_AT, lambda_GT) with p10 = lambda_GC and
pi fixed at its starting value.
"""
import math
import time
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

from . import model as M

FREE = ("q1", "q2", "q3", "q4", "q5", "q6", "siteGammaShape", "lambdazeroweight", "lambdaGC", "lambdaAT",
        "lambdaGT")
NFREE = len(FREE)


# ---------------------------------------------------------------------------
# parameter vectors
# ---------------------------------------------------------------------------
def theta_from_p15(p15):
    p = np.asarray(p15, np.float64)
    return np.array([p[3], p[4], p[5], p[6], p[7], p[8], p[10], p[14], p[0], p[1], p[2]])


def p15_from_theta(theta, pi3):
    t = np.asarray(theta, np.float64)
    return np.array([t[8], t[9], t[10], t[0], t[1], t[2], t[3], t[4], t[5], t[8], t[6], pi3[0], pi3[1], pi3[2],
                     t[7]])


def isvalid_theta(t):
    """src/MCMC.jl:292-305 on the free parameters (shape_GC = lambda_GC >= 1, ...)."""
    t = np.asarray(t)
    return bool(np.all(t[0:6] >= 0.0) and t[6] > 0.0 and 0.0 <= t[7] <= 1.0 and np.all(t[8:11] >= 1.0))


def to_z(t):
    """Unconstrained coordinates: log for rates and shape, logit for the
    weight, log(lambda - 1) for the lambdas."""
    t = np.asarray(t, np.float64)
    z = np.empty(NFREE)
    z[0:7] = np.log(t[0:7])
    z[7] = math.log(t[7]) - math.log1p(-t[7])
    z[8:11] = np.log(t[8:11] - 1.0)
    return z


def from_z(z):
    z = np.asarray(z, np.float64)
    t = np.empty(NFREE)
    t[0:7] = np.exp(z[0:7])
    t[7] = 1.0 / (1.0 + math.exp(-z[7]))
    t[8:11] = 1.0 + np.exp(z[8:11])
    return t


def log_jacobian(z):
    """log |d theta / d z|."""
    z = np.asarray(z, np.float64)
    s = float(np.sum(z[0:7]) + np.sum(z[8:11]))
    s += -abs(z[7]) - 2.0 * math.log1p(math.exp(-abs(z[7])))  # log sigma(z)(1 - sigma(z))
    return s


# ---------------------------------------------------------------------------
# target
# ---------------------------------------------------------------------------
class Target:
    """log posterior = computeprior + Z (src/FARCE.jl:2347-2352) on the GPU."""

    def __init__(self, dataset, pi3, maxbasepairdistance, ctx=None, gapcutoff=1.0):
        from . import api
        self.api = api
        self.ds = dataset
        self.pi3 = np.asarray(pi3, np.float64)
        self.W = maxbasepairdistance
        self.ctx = ctx or api.get_context()
        self.gapcutoff = gapcutoff
        self.evals = 0
        self.launches = 0

    def __call__(self, theta):
        if not isvalid_theta(theta):
            return -math.inf
        p15 = p15_from_theta(theta, self.pi3)
        if p15[11] + p15[12] + p15[13] >= 0.95:  # src/MESSI.jl:287-289
            return -math.inf
        params = M.getparams(p15, self.ds.branchlengths)
        self.evals += 1
        ll = self.api.computestructureintegratedlikelihood(self.ds, params, self.W, ctx=self.ctx,
                                                            gapcutoff=self.gapcutoff)
        self.launches += self.ctx.last_launches()
        return ll if math.isfinite(ll) else -math.inf


# ---------------------------------------------------------------------------
# plain proposal: move 8 (src/MCMC.jl:1543-1597) + gettunedparams (:393-449)
# ---------------------------------------------------------------------------
def tuning_vector(theta):
    """gettuningvector (src/MCMC.jl:307-326); entries 10/12/14 are the gamma
    scale, which getparams resets to 1.0."""
    t = theta
    return np.array([t[0], t[1], t[2], t[3], t[4], t[5], t[6], t[7], t[8], 1.0, t[9], 1.0, t[10], 1.0])


def theta_from_tuning(tv):
    """settuningparams (src/MCMC.jl:330-370) followed by the getparams round trip."""
    return np.array([tv[0], tv[1], tv[2], tv[3], tv[4], tv[5], tv[6], tv[7], tv[8], tv[10], tv[12]])


def gettunedparams(rng, current, tuningvectors, mask, covarScale=1.0, C=0.005):
    d = len(current)
    d2 = int(np.sum(mask))
    r = rng.random()
    e = np.eye(d) * (0.00025 if r < 0.25 else 0.0025 if r < 0.5 else 0.0075 if r < 0.75 else 0.025)
    n = len(tuningvectors)
    if n < 16 * d:
        e[7, 7] *= 0.25
        if n % 2 == 0:
            cov = 2.38 * 2.38 * e / d2 / 2.0
            return current + rng.multivariate_normal(np.zeros(d), cov) * mask
        cov = 2.38 * 2.38 * e / d / 2.0
        return current + rng.multivariate_normal(np.zeros(d), cov)
    eyemat = np.eye(d) * 0.0001 / d2
    reg = 0.001 * np.eye(d) / n
    hist = np.asarray(tuningvectors[max(0, n // 2 - 1):n])
    cov = 2.38 * 2.38 * np.cov(hist.T) / d2
    r1 = rng.multivariate_normal(np.zeros(d), eyemat) * mask
    r2 = rng.multivariate_normal(np.zeros(d), (cov + reg) * covarScale) * mask
    return C * (current + r1) + (1.0 - C) * (current + r2)


class PlainProposal:
    """Symmetric adaptive random walk: Hastings correction 0."""

    name = "plain"

    def __init__(self, max_tuning_iter=10000, tuning_scale=1.0):
        self.tuningvectors: List[np.ndarray] = []
        self.max_tuning_iter = max_tuning_iter
        self.scale = tuning_scale

    def propose(self, rng, theta):
        cur = tuning_vector(theta)
        r = rng.random()
        mask = np.zeros(14)
        if r < 0.3:
            for i in rng.permutation([7, 8, 9, 10, 12])[:2]:
                mask[i] = 1
        elif r < 0.6:
            mask[:] = 1
        elif r < 0.8:
            mask[[7, 8, 9, 10, 12]] = 1
        elif r < 0.9:
            mask[0:7] = 1
        else:
            mask[rng.permutation(6)[:3]] = 1
        new = gettunedparams(rng, cur, self.tuningvectors, mask, self.scale)
        return theta_from_tuning(new), 0.0

    def observe(self, it, theta):
        if it < self.max_tuning_iter:
            self.tuningvectors.append(tuning_vector(theta))


# ---------------------------------------------------------------------------
# learned proposal
# ---------------------------------------------------------------------------
def alignment_summaries(ds, n=32):
    """32 fixed statistics of the alignment fed to the network with the state:
    gap statistics, nucleotide composition, per-column diversity quantiles,
    size terms."""
    m = ds.masks
    N, L = m.shape
    single = np.isin(m, (1, 2, 4, 8))
    comp = [float(np.mean(m == v)) for v in (1, 2, 4, 8, 15)]
    gap = ds.gapfrequency
    # per-column number of distinct characters and fraction of the majority one
    distinct = np.array([len(np.unique(m[:, j])) for j in range(L)], np.float64)
    major = np.array([np.max(np.bincount(m[:, j], minlength=16)) / N for j in range(L)])
    q = np.linspace(0.05, 0.95, 10)
    feats = comp + [float(gap.mean()), float(gap.std()), float(np.mean(gap > 0.5)), float(single.mean())]
    feats += list(np.quantile(distinct, q) / 16.0) + list(np.quantile(major, q))
    feats += [math.log(N) / 8.0, math.log(L) / 10.0, float(np.mean(np.diff(ds.branchlengths[1:]) ** 2) if ds.numnodes > 2
                                                          else 0.0), float(np.sum(ds.branchlengths))]
    feats = np.asarray(feats[:n], np.float64)
    if len(feats) < n:
        feats = np.concatenate([feats, np.zeros(n - len(feats))])
    return feats


class LearnedProposal:
    """Gaussian-mixture proposal in z-space from the GPU MLP."""

    name = "learned"

    def __init__(self, summaries, ncomp=4, width=256, seed=1, ctx=None, lr=2e-3, inflate=1.25, net=None,
                 local_w=0.25, wide_w=0.1, wide_scale=2.0):
        self.summ = np.asarray(summaries, np.float64)
        self.K = ncomp
        self.D = NFREE
        self.in_dim = NFREE + 1 + len(self.summ)  # the 12 parameters (p10 tied) + summaries
        if net is None:
            from . import api
            net = api.MLP(self.in_dim, width, ncomp, self.D, seed=seed, ctx=ctx)
        self.net = net
        self.lr = lr
        # proposal scales are the fitted ones times `inflate` (in both the
        # draw and the density), which keeps a fit to an under-dispersed
        # burn-in sample from starving the tails
        self.log_inflate = math.log(inflate)
        self.local_w = float(local_w)
        self.wide_w = float(wide_w)
        self.wide_scale = float(wide_scale)
        # affine whitening z = zmu + Lw @ zn (Lw: Cholesky factor of the
        # covariance of the recent burn-in states), so the diagonal mixture
        # works in coordinates where the posterior is close to isotropic
        self.zmu = np.zeros(self.D)
        self.Lw = np.eye(self.D)
        self.Lw_inv = np.eye(self.D)
        self.logdet = 0.0
        self.train_time = 0.0
        self.train_steps = 0
        self.frozen = False

    def _inputs(self, Z):
        Z = np.atleast_2d(Z)
        zn = self._whiten(Z)
        tied = zn[:, 8:9]  # p10 = lambda_GC
        return np.hstack([zn, tied, np.tile(self.summ, (Z.shape[0], 1))])

    def _whiten(self, Z):
        return (np.atleast_2d(Z) - self.zmu) @ self.Lw_inv.T

    def _mixture(self, head, zn_from):
        """Mixture over the K network components plus one local component
        N(zn_from, (2.38^2 / D) I) of weight `local_w` (the adaptive-Metropolis
        step in whitened coordinates), which keeps the chain moving where the
        fitted components are poor.  Both directions of the Metropolis-Hastings
        ratio evaluate this same density."""
        K, D = self.K, self.D
        logits = head[:, :K].astype(np.float64)
        mu = head[:, K:K + K * D].astype(np.float64).reshape(-1, K, D)
        ls = np.clip(head[:, K + K * D:].astype(np.float64).reshape(-1, K, D), -7.0, 5.0) + self.log_inflate
        lw = logits - np.logaddexp.reduce(logits, axis=1, keepdims=True) + math.log1p(-self.local_w - self.wide_w)
        n = head.shape[0]
        lw = np.hstack([lw, np.full((n, 1), math.log(self.local_w)), np.full((n, 1), math.log(self.wide_w))])
        mu = np.concatenate([mu, np.atleast_2d(zn_from)[:, None, :], np.zeros((n, 1, D))], axis=1)
        ls = np.concatenate([ls, np.full((n, 1, D), math.log(2.38 / math.sqrt(D))),
                             np.full((n, 1, D), math.log(self.wide_scale))], axis=1)
        return lw, mu, ls

    def _logq_norm(self, lw, mu, ls, zn):
        diff = zn[:, None, :] - mu
        lp = lw + np.sum(-0.5 * (diff * np.exp(-ls)) ** 2 - ls, axis=2) - 0.91893853320467274 * self.D
        return np.logaddexp.reduce(lp, axis=1)

    def logq(self, z_to, z_from):
        """log q(z_to | z_from) in z coordinates (includes the normalisation
        scale of the whitened space)."""
        head = self.net.forward(self._inputs(z_from))
        lw, mu, ls = self._mixture(head, self._whiten(z_from))
        return self._logq_norm(lw, mu, ls, self._whiten(z_to)) - self.logdet

    def propose(self, rng, theta):
        z = to_z(theta)
        head = self.net.forward(self._inputs(z))
        lw, mu, ls = self._mixture(head, self._whiten(z))
        w = np.exp(lw[0])
        k = rng.choice(len(w), p=w / w.sum())
        zn_new = mu[0, k] + np.exp(ls[0, k]) * rng.standard_normal(self.D)
        z_new = self.zmu + self.Lw @ zn_new
        fwd = self._logq_norm(lw, mu, ls, zn_new[None, :])[0] - self.logdet
        rev = self.logq(z, z_new)[0]
        # target density in z-space carries the Jacobian of theta(z)
        hastings = rev - fwd + log_jacobian(z_new) - log_jacobian(z)
        return from_z(z_new), hastings

    def fit(self, rng, Zbuf, steps=200, batch=256):
        """Train on the chain's states: inputs are random states, targets other
        random states, so q(. | z) learns the chain's stationary distribution."""
        if self.frozen or len(Zbuf) < 16:
            return None
        t0 = time.perf_counter()
        Z = np.asarray(Zbuf)
        Z = Z[len(Z) // 2:]  # the recent half: the early burn-in is a transient
        self.zmu = Z.mean(axis=0)
        cov = np.cov(Z.T) + 1e-8 * np.eye(self.D)
        cov += np.diag(np.maximum(np.diag(cov), 1e-6) * 1e-3)
        self.Lw = np.linalg.cholesky(cov)
        self.Lw_inv = np.linalg.inv(self.Lw)
        self.logdet = float(np.sum(np.log(np.diag(self.Lw))))
        loss = None
        for _ in range(steps):
            a = Z[rng.integers(0, len(Z), batch)]
            b = Z[rng.integers(0, len(Z), batch)]
            loss = self.net.train_step(self._inputs(a), self._whiten(b), lr=self.lr)
            self.train_steps += 1
        self.train_time += time.perf_counter() - t0
        return loss


# ---------------------------------------------------------------------------
# chain
# ---------------------------------------------------------------------------
@dataclass
class ChainResult:
    samples: np.ndarray          # [n, 11] post-burn-in states
    logpost: np.ndarray
    accept: dict
    seconds: float               # wall time of the whole run (training included)
    sample_seconds: float        # wall time of the post-burn-in part
    evals: int
    extra: dict = field(default_factory=dict)


def run_chain(target, theta0, iterations, burnin, proposal="plain", seed=1, learned: Optional[LearnedProposal] = None,
              learned_prob=0.9, fit_every=100, fit_steps=150, warm_plain=None, callback=None):
    """Metropolis-Hastings (src/MCMC.jl:1666): accept with probability
    min(1, exp(ll' - ll + log Hastings correction))."""
    rng = np.random.default_rng(seed)
    plain = PlainProposal()
    theta = np.asarray(theta0, np.float64)
    ll = target(theta)
    if not math.isfinite(ll):
        raise ValueError("starting point has zero posterior density")
    samples, lps = [], []
    acc = {"plain": [0, 0], "learned": [0, 0]}
    zbuf = []
    warm_plain = burnin // 2 if warm_plain is None else warm_plain
    t_start = time.perf_counter()
    t_sample = None
    for it in range(iterations):
        if it == burnin:
            t_sample = time.perf_counter()
            if learned is not None:
                learned.frozen = True
        use_learned = (proposal == "learned" and learned is not None and it >= warm_plain
                       and rng.random() < learned_prob)
        prop = learned if use_learned else plain
        theta_new, hastings = prop.propose(rng, theta)
        ll_new = target(theta_new) if isvalid_theta(theta_new) else -math.inf
        key = prop.name
        acc[key][1] += 1
        if math.isfinite(ll_new) and math.log(rng.random() + 1e-300) < (ll_new - ll) + hastings:
            theta, ll = theta_new, ll_new
            acc[key][0] += 1
        plain.observe(it, theta)
        if proposal == "learned" and learned is not None and it < burnin:
            zbuf.append(to_z(theta))
            if it + 1 >= fit_every and (it + 1) % fit_every == 0:
                learned.fit(rng, zbuf, steps=fit_steps)
        if it >= burnin:
            samples.append(theta.copy())
            lps.append(ll)
        if callback:
            callback(it, theta, ll)
    t_end = time.perf_counter()
    extra = {}
    if learned is not None:
        extra = {"train_seconds": learned.train_time, "train_steps": learned.train_steps}
    return ChainResult(samples=np.asarray(samples), logpost=np.asarray(lps),
                       accept={k: (v[0] / v[1] if v[1] else None, v[1]) for k, v in acc.items()},
                       seconds=t_end - t_start, sample_seconds=t_end - (t_sample or t_end),
                       evals=getattr(target, "evals", 0), extra=extra)


# ---------------------------------------------------------------------------
# effective sample size and Monte Carlo standard error
# ---------------------------------------------------------------------------
def autocorr(x):
    x = np.asarray(x, np.float64) - np.mean(x)
    n = len(x)
    if n < 2 or np.allclose(x, 0.0):
        return np.ones(1)
    f = np.fft.rfft(x, 2 * n)
    ac = np.fft.irfft(f * np.conj(f))[:n]
    return ac / ac[0]


def ess(x):
    """Geyer's initial monotone sequence estimator."""
    x = np.asarray(x, np.float64)
    n = len(x)
    if n < 4:
        return float(n)
    rho = autocorr(x)
    if len(rho) < 2:
        return 0.0
    gam = []
    for k in range(0, n // 2 - 1):
        g = rho[2 * k] + rho[2 * k + 1]
        if g <= 0:
            break
        gam.append(g)
    if not gam:
        return float(n)
    gam = np.minimum.accumulate(np.asarray(gam))
    tau = -1.0 + 2.0 * np.sum(gam)
    return float(n / max(tau, 1e-12))


def mcse(x, nbatch=None):
    """Batch-means Monte Carlo standard error of the mean."""
    x = np.asarray(x, np.float64)
    n = len(x)
    b = nbatch or max(2, int(math.sqrt(n)))
    size = n // b
    if size < 1:
        return float("nan")
    means = x[:size * b].reshape(b, size).mean(axis=1)
    return float(means.std(ddof=1) / math.sqrt(b))
