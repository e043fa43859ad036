"""CPU: the sampler logic (gliomauq_gb300/mcmc.py) on targets with known
answers -- ESS of AR(1) chains, and RWM / MALA on a Gaussian posterior
stub with the solver's call signature."""
import numpy as np

from gliomauq_gb300 import mcmc


def test_ess_of_independent_and_ar1_chains():
    rng = np.random.default_rng(0)
    iid = rng.standard_normal((4000, 8, 1))
    e = mcmc.ess(iid)[0]
    assert 0.8 * 32000 < e < 1.25 * 32000
    phi = 0.9
    x = np.zeros((20000, 4, 1))
    for t in range(1, x.shape[0]):
        x[t] = phi * x[t - 1] + rng.standard_normal((4, 1))
    exp = 80000 * (1 - phi) / (1 + phi)
    assert 0.7 * exp < mcmc.ess(x)[0] < 1.3 * exp


class GaussianStub:
    """Posterior with the solver's interface: N(mu, diag(sd^2)) inside a box."""

    def __init__(self):
        self.mu = np.array([1.2e-3, 0.1, 30.0, 32.0, 31.0, 300.0])
        self.sd = np.array([1e-4, 0.01, 1.0, 1.0, 1.0, 20.0])
        self.prior = mcmc.Prior(lo=self.mu - 20 * self.sd, hi=self.mu + 20 * self.sd,
                                seed_mask=np.ones((64, 64, 64), dtype=bool))
        self.solves = 0

    def loglik(self, th, with_grad):
        th = np.atleast_2d(th)
        self.solves += th.shape[0]
        z = (th - self.mu) / self.sd
        lp = self.prior.logp(th)
        return -0.5 * np.sum(z * z, axis=1) + lp, -(th - self.mu) / self.sd ** 2


def test_mala_and_rwm_recover_a_gaussian():
    rng = np.random.default_rng(1)
    post = GaussianStub()
    th0 = post.mu + post.sd * rng.standard_normal((16, 6))
    r = mcmc.mala(post, th0, 1500, 0.05, rng, burn=300)
    s = r.samples[300:].reshape(-1, 6)
    assert 0.4 < r.accept < 0.75
    assert np.all(np.abs(s.mean(axis=0) - post.mu) < 0.15 * post.sd)
    assert np.all(np.abs(s.std(axis=0) / post.sd - 1) < 0.15)
    assert np.all(mcmc.ess(r.samples[300:]) > 300)
    r2 = mcmc.rwm(post, th0, 3000, 0.01, rng, burn=500)
    s2 = r2.samples[500:].reshape(-1, 6)
    assert 0.1 < r2.accept < 0.4
    assert np.all(np.abs(s2.mean(axis=0) - post.mu) < 0.3 * post.sd)
