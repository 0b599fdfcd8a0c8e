"""MCMC host logic (no GPU): transforms, the restated move-8 proposal, ESS and MCSE."""
import math

import numpy as np

from messi_gb300 import mcmc


def test_transform_round_trip_and_jacobian():
    rng = np.random.default_rng(0)
    for _ in range(20):
        theta = np.concatenate([rng.uniform(0.05, 6.0, 6), [rng.uniform(0.2, 3.0)], [rng.uniform(0.05, 0.95)],
                                rng.uniform(1.01, 5.0, 3)])
        z = mcmc.to_z(theta)
        np.testing.assert_allclose(mcmc.from_z(z), theta, rtol=1e-12)
        h = 1e-6
        num = 0.0
        for k in range(mcmc.NFREE):
            dz = np.zeros(mcmc.NFREE)
            dz[k] = h
            num += math.log(abs((mcmc.from_z(z + dz)[k] - mcmc.from_z(z - dz)[k]) / (2 * h)))
        assert abs(num - mcmc.log_jacobian(z)) < 1e-5


def test_p15_round_trip_ties_gamma_shape():
    theta = np.array([1.7, 4.4, 1.6, 0.48, 5.8, 0.71, 0.61, 0.5, 2.5, 3.0, 1.5])
    pi3 = np.array([0.23, 0.26, 0.24])
    p15 = mcmc.p15_from_theta(theta, pi3)
    assert p15[9] == theta[8]  # lambda gamma shape tied to lambda_GC (settuningparams)
    np.testing.assert_array_equal(mcmc.theta_from_p15(p15), theta)
    assert mcmc.isvalid_theta(theta)
    bad = theta.copy()
    bad[9] = 0.9
    assert not mcmc.isvalid_theta(bad)


def test_move8_proposal_is_centred_and_masked():
    rng = np.random.default_rng(3)
    theta = np.array([1.7, 4.4, 1.6, 0.48, 5.8, 0.71, 0.61, 0.5, 2.5, 3.0, 1.5])
    cur = mcmc.tuning_vector(theta)
    # even history length: only masked entries move
    mask = np.zeros(14)
    mask[[0, 3]] = 1
    for _ in range(50):
        new = mcmc.gettunedparams(rng, cur, [cur] * 10, mask)
        assert np.all(new[mask == 0] == cur[mask == 0])
    # adaptive branch: proposals are centred on the current point (symmetric)
    hist = [cur + rng.normal(0, 0.05, 14) for _ in range(400)]
    draws = np.array([mcmc.gettunedparams(rng, cur, hist, np.ones(14)) for _ in range(3000)])
    se = draws.std(axis=0) / math.sqrt(len(draws))
    assert np.all(np.abs(draws.mean(axis=0) - cur) < 5 * se + 1e-12)
    p = mcmc.PlainProposal()
    t2, h = p.propose(rng, theta)
    assert h == 0.0 and t2.shape == (11,)


def test_ess_on_ar1():
    rng = np.random.default_rng(5)
    n, phi = 40000, 0.5
    x = np.zeros(n)
    for i in range(1, n):
        x[i] = phi * x[i - 1] + rng.standard_normal()
    tau = (1 + phi) / (1 - phi)
    assert abs(mcmc.ess(x) - n / tau) < 0.15 * n / tau
    iid = rng.standard_normal(n)
    assert mcmc.ess(iid) > 0.8 * n
    # MCSE of the mean of an AR(1): sd * sqrt(tau / n)
    expected = math.sqrt(1 / (1 - phi ** 2)) * math.sqrt(tau / n)
    assert abs(mcmc.mcse(x) - expected) < 0.35 * expected


class _ZeroHead:
    """Stand-in for the proposal network: every head is zero, so the learned
    proposal is the whitened Gaussian N(zmu, inflate^2 * Cov) of the burn-in."""

    def __init__(self, K, D):
        self.width = K + 2 * K * D

    def forward(self, x):
        return np.zeros((np.atleast_2d(x).shape[0], self.width), np.float32)

    def train_step(self, x, t, lr=None):
        return 0.0


def test_whitened_learned_proposal_is_exact_on_a_correlated_target():
    rng = np.random.default_rng(8)
    D = mcmc.NFREE
    A = rng.normal(size=(D, D))
    cov = 0.02 * (A @ A.T / D + 0.1 * np.eye(D))
    icov = np.linalg.inv(cov)
    m = np.array([0.5, 1.4, 0.5, -0.7, 1.7, -0.3, -0.5, 0.0, 0.4, 0.7, -0.7])

    def target(theta):
        if not mcmc.isvalid_theta(theta) or theta[7] <= 0.0 or theta[7] >= 1.0:
            return -math.inf
        z = mcmc.to_z(theta)
        d = z - m
        return float(-0.5 * d @ icov @ d - mcmc.log_jacobian(z))

    lp = mcmc.LearnedProposal(np.zeros(4), ncomp=2, net=_ZeroHead(2, D))
    res = mcmc.run_chain(target, mcmc.from_z(m + 0.1), 15000, 5000, proposal="learned", seed=4, learned=lp,
                         fit_every=250, fit_steps=1)
    Z = np.array([mcmc.to_z(t) for t in res.samples])
    assert res.accept["learned"][0] > 0.2
    sd = np.sqrt(np.diag(cov))
    for k in range(D):
        assert abs(Z[:, k].mean() - m[k]) < 5 * mcmc.mcse(Z[:, k]) + 0.02 * sd[k]
    np.testing.assert_allclose(np.cov(Z.T), cov, atol=0.25 * np.max(np.diag(cov)))
