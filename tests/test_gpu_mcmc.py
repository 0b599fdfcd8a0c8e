"""HP3 on the GPU: the proposal network's kernels against the FP64 oracle,
its training, and the learned Metropolis-Hastings proposal (exactness on a
known target, gain over the plain move, a chain on the real likelihood)."""
import math

import numpy as np
import pytest

from oracle import mlp_ref

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def api():
    from messi_gb300 import api as _api
    return _api


def test_mlp_gradients_match_oracle(api):
    rng = np.random.default_rng(3)
    nin, H, K, D = 44, 256, 4, 11
    net = api.MLP(nin, H, K, D, seed=7)
    p = net.get_params().astype(np.float64)
    x = rng.normal(size=(96, nin))
    t = rng.normal(size=(96, D))
    loss, g = net.gradients(x, t)
    loss_ref, g_ref = mlp_ref.gradients(p, x, t, nin, H, K, D, bf16=True)
    assert abs(loss - loss_ref) <= 1e-4 * abs(loss_ref)
    assert np.linalg.norm(g - g_ref) <= 1e-3 * np.linalg.norm(g_ref)
    # against unrounded FP64 maths: BF16 weights/activations cost ~1e-2
    loss64, g64 = mlp_ref.gradients(p, x, t, nin, H, K, D, bf16=False)
    assert np.linalg.norm(g - g64) <= 5e-2 * np.linalg.norm(g64)
    cos = float(g @ g64 / (np.linalg.norm(g) * np.linalg.norm(g64)))
    assert cos > 0.999
    # forward head equals the oracle's
    y = net.forward(x[:8])
    f = mlp_ref.forward(p, x[:8], nin, H, K + 2 * K * D, bf16=True)
    np.testing.assert_allclose(y, f["y"], rtol=1e-3, atol=1e-4)


def test_mlp_training_fits_a_gaussian(api):
    rng = np.random.default_rng(4)
    nin, D = 16, 3
    net = api.MLP(nin, 64, 2, D, seed=11)
    mu = np.array([1.0, -2.0, 0.5])
    sd = np.array([0.3, 1.0, 0.6])
    first = None
    for step in range(400):
        x = rng.normal(size=(128, nin))
        t = mu + sd * rng.standard_normal((128, D))
        loss = net.train_step(x, t, lr=3e-3)
        first = loss if first is None else first
    assert loss < first - 1.0
    head = net.forward(rng.normal(size=(64, nin))).astype(np.float64)
    K = 2
    w = np.exp(head[:, :K] - np.logaddexp.reduce(head[:, :K], axis=1, keepdims=True))
    means = head[:, K:K + K * D].reshape(-1, K, D)
    mean = np.einsum("bk,bkd->bd", w, means).mean(axis=0)
    assert np.all(np.abs(mean - mu) < 0.25)


class ToyTarget:
    """theta whose z = to_z(theta) is N(m, diag(s^2)) (cheap, known moments)."""

    def __init__(self):
        from messi_gb300 import mcmc
        self.mcmc = mcmc
        self.m = np.array([0.5, 1.4, 0.5, -0.7, 1.7, -0.3, -0.5, 0.0, 0.4, 0.7, -0.7])
        self.s = np.array([0.2, 0.1, 0.25, 0.3, 0.1, 0.3, 0.15, 0.4, 0.3, 0.2, 0.5])
        self.evals = 0

    def __call__(self, theta):
        if not self.mcmc.isvalid_theta(theta) or theta[7] <= 0.0 or theta[7] >= 1.0:
            return -math.inf
        z = self.mcmc.to_z(theta)
        self.evals += 1
        return float(-0.5 * np.sum(((z - self.m) / self.s) ** 2) - self.mcmc.log_jacobian(z))


def test_learned_proposal_is_exact_and_beats_the_plain_move(api):
    from messi_gb300 import mcmc
    tgt = ToyTarget()
    theta0 = mcmc.from_z(tgt.m + 0.5 * tgt.s)
    summ = np.linspace(-1, 1, 32)
    n, burn = 20000, 6667
    plain = mcmc.run_chain(tgt, theta0, n, burn, proposal="plain", seed=1)
    learned = mcmc.LearnedProposal(summ, seed=5)
    lrn = mcmc.run_chain(tgt, theta0, n, burn, proposal="learned", seed=2, learned=learned, fit_every=333,
                         fit_steps=60)
    for res in (plain, lrn):
        Z = np.array([mcmc.to_z(t) for t in res.samples])
        for k in range(mcmc.NFREE):
            se = mcmc.mcse(Z[:, k])
            assert abs(Z[:, k].mean() - tgt.m[k]) < 5 * se + 0.02 * tgt.s[k], (res.accept, k)
    ess_p = np.array([mcmc.ess(np.array([mcmc.to_z(t) for t in plain.samples])[:, k]) for k in range(mcmc.NFREE)])
    ess_l = np.array([mcmc.ess(np.array([mcmc.to_z(t) for t in lrn.samples])[:, k]) for k in range(mcmc.NFREE)])
    assert lrn.accept["learned"][0] > 0.3
    assert np.median(ess_l) >= 3.0 * np.median(ess_p), (np.median(ess_l), np.median(ess_p))


def test_chain_on_the_gpu_likelihood(api, c1):
    from messi_gb300 import mcmc
    ds = c1.dataset
    tgt = mcmc.Target(ds, c1.params15[11:14], c1.W)
    theta0 = mcmc.theta_from_p15(c1.params15)
    theta0[8] = max(theta0[8], 1.05)
    res = mcmc.run_chain(tgt, theta0, 40, 10, proposal="plain", seed=3)
    assert res.samples.shape == (30, mcmc.NFREE) and np.all(np.isfinite(res.logpost))
    learned = mcmc.LearnedProposal(mcmc.alignment_summaries(ds), seed=9)
    res2 = mcmc.run_chain(tgt, theta0, 60, 40, proposal="learned", seed=4, learned=learned, fit_every=20,
                          fit_steps=20, warm_plain=20)
    assert res2.samples.shape == (20, mcmc.NFREE) and np.all(np.isfinite(res2.logpost))
    assert res2.accept["learned"][1] > 0
    assert tgt.launches > 0
