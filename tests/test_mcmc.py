"""CPU: the sampler logic (gliomauq_gb300/mcmc.py) on targets with known
answers -- ESS of AR(1) chains, and RWM / MALA on a Gaussian posterior
stub with the solver's call signature."""
import numpy as np
import pytest

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


class BiasedSurrogateStub:
    """Surrogate with the library binding's interface whose log L is the
    Gaussian stub's with a shifted mean, a 30% wider spread and a constant
    offset: delayed acceptance must still sample the stub exactly."""

    def __init__(self, post):
        self.post = post
        self.batch_max = 8
        self.calls = 0

    def loglik(self, samples):
        th = np.asarray(samples, dtype=np.float64)
        self.calls += 1
        assert th.shape[0] <= self.batch_max
        z = (th - self.post.mu - 0.5 * self.post.sd) / (1.3 * self.post.sd)
        ll = -0.5 * np.sum(z * z, axis=1) - 1234.5
        return dict(loglik=[dict(total=v) for v in ll])


def test_delayed_acceptance_targets_the_exact_posterior():
    rng = np.random.default_rng(3)
    post = GaussianStub()
    sur = BiasedSurrogateStub(post)
    spost = mcmc.SurrogatePosterior(sur, post.prior)
    th0 = post.mu + post.sd * rng.standard_normal((32, 6))
    r = mcmc.da(post, spost, th0, 1200, 0.02, rng, inner=6, burn=200)
    s = r.samples[200:].reshape(-1, 6)
    assert np.all(np.abs(s.mean(axis=0) - post.mu) < 0.15 * post.sd)
    assert np.all(np.abs(s.std(axis=0) / post.sd - 1) < 0.15)
    h = r.history
    assert 0.15 < h["stage1_accept"] < 0.5
    assert 0.2 < h["stage2_accept"] <= 1.0
    # one solver call per generation for the moved chains, `inner` surrogate
    # passes in batches of batch_max
    assert sur.calls >= 6 * 1200 * 32 // 8
    assert post.solves <= 32 * 1201
    # with adaptation the target is still exact
    r = mcmc.da(post, spost, th0, 1200, 0.02, rng, inner=6, burn=200, chol=np.diag(post.sd),
                adapt=True)
    s = r.samples[200:].reshape(-1, 6)
    assert np.all(np.abs(s.mean(axis=0) - post.mu) < 0.15 * post.sd)
    assert np.all(np.abs(s.std(axis=0) / post.sd - 1) < 0.15)
    assert np.all(mcmc.rhat(r.samples[200:]) < 1.05)


def test_burn_in_resets_stranded_chains():
    """A quarter of the chains start 10 sd away (≈ 150 nats below the
    bulk): at the rebuild points of burn-in they are moved onto copies of
    chains in the bulk, and the post-burn-in population samples the
    posterior; reset_stranded=False makes no resets."""
    rng = np.random.default_rng(5)
    post = GaussianStub()
    sur = BiasedSurrogateStub(post)
    spost = mcmc.SurrogatePosterior(sur, post.prior)
    th0 = post.mu + post.sd * rng.standard_normal((32, 6))
    th0[:8] = post.mu + 10.0 * post.sd * np.array([1, -1, 1, -1, 1, -1])
    kw = dict(inner=6, burn=60, chol=np.diag(post.sd), adapt=True, rebuild_every=10)
    r = mcmc.da(post, spost, th0, 400, 0.02, rng, **kw)
    assert r.history["stranded_resets"] >= 8
    s = r.samples[60:]
    z = np.abs((s - post.mu) / post.sd).max(axis=(0, 2))  # per chain, after burn-in
    assert np.all(z < 6.0), z
    assert np.all(np.abs(s.reshape(-1, 6).mean(axis=0) - post.mu) < 0.3 * post.sd)
    r0 = mcmc.da(post, spost, th0, 61, 0.02, np.random.default_rng(5), reset_stranded=False, **kw)
    assert r0.history["stranded_resets"] == 0


class TiltedSurrogate:
    """Exact log pi plus a linear tilt; rebuild() scales the tilt by
    `factor` (below 1: a better surrogate, above 1: a worse one);
    state()/restore() as the affine surrogate's."""

    def __init__(self, post, tilt, factor):
        self.post, self.tilt, self.factor = post, np.asarray(tilt, dtype=float), factor
        self.evals = 0

    def logpost(self, th):
        th = np.atleast_2d(th)
        self.evals += th.shape[0]
        lp, _ = self.post.loglik(th, False)
        return lp + ((th - self.post.mu) / self.post.sd) @ self.tilt

    def rebuild(self, centre, steps):
        self.tilt = self.tilt * self.factor

    def state(self):
        return self.tilt.copy()

    def restore(self, st):
        self.tilt = st.copy()


@pytest.mark.parametrize("factor,kept", [(0.5, 5), (2.0, 0)])
def test_surrogate_rebuilds_are_kept_only_when_they_help(factor, kept):
    rng = np.random.default_rng(9)
    post = GaussianStub()
    tilt = np.array([0.3, -0.2, 0.1, 0.0, 0.2, -0.1])
    sur = TiltedSurrogate(post, tilt, factor)
    th0 = post.mu + post.sd * rng.standard_normal((32, 6))
    r = mcmc.da(post, sur, th0, 40, 0.02, rng, inner=4, burn=30, chol=np.diag(post.sd),
                adapt=True, rebuild_every=5)
    assert r.history["rebuilds_tried"] == 5
    assert r.history["rebuilds_kept"] == kept
    expect = tilt * factor ** kept
    assert np.allclose(sur.tilt, expect)


class InvariantStub(GaussianStub):
    """Likelihood that depends on (log rho T, log Dw/rho, x0, y0, z0) only
    (Gaussian there), prior box on theta: the tumour model's symmetry."""

    def __init__(self):
        super().__init__()
        self.prior = mcmc.Prior(lo=np.array([2e-4, 0.01, 20, 20, 20, 100.0]),
                                hi=np.array([2.5e-3, 0.2, 44, 44, 44, 500.0]),
                                seed_mask=np.ones((64, 64, 64), dtype=bool))
        self.c = np.array([np.log(0.15 * 260.0), np.log(6e-4 / 0.15), 30.0, 32.0, 31.0])
        self.s = np.array([0.01, 0.02, 0.5, 0.5, 0.5])

    def inv(self, th):
        th = np.atleast_2d(th)
        return np.stack([np.log(th[:, 1] * th[:, 5]), np.log(th[:, 0] / th[:, 1]),
                         th[:, 2], th[:, 3], th[:, 4]], axis=1)

    def loglik(self, th, with_grad):
        th = np.atleast_2d(th)
        self.solves += th.shape[0]
        z = (self.inv(th) - self.c) / self.s
        return -0.5 * np.sum(z * z, axis=1) + self.prior.logp(th), None


class InvariantSurrogate:
    """The invariant stub's log L with a shifted centre (a biased screen)."""
    batch_max = 16

    def __init__(self, post):
        self.post = post

    def loglik(self, samples):
        th = np.asarray(samples, dtype=np.float64)
        z = (self.post.inv(th) - self.post.c - 0.3 * self.post.s) / (1.2 * self.post.s)
        return dict(loglik=[dict(total=v) for v in -0.5 * np.sum(z * z, axis=1)])


def test_delayed_acceptance_with_symmetry_axis_redraw():
    rng = np.random.default_rng(8)
    base = InvariantStub()
    lc = mcmc.LogCoords(base, A=mcmc.INVARIANT_MAP)
    sp = lc.surrogate(mcmc.SurrogatePosterior(InvariantSurrogate(base), base.prior))
    v_c = np.concatenate([[np.log(0.15)], base.c])
    v0 = v_c + np.concatenate([[0.0], base.s]) * rng.standard_normal((32, 6))
    v0 = lc.prior.redraw_axis(v0, 0, rng)
    chol = np.diag(np.concatenate([[0.1], base.s]))
    r = mcmc.da(lc, sp, v0, 1500, 1.0, rng, inner=6, burn=300, chol=chol, adapt=True, axis=0)
    v = r.samples[300:]
    flat = v.reshape(-1, 6)
    # seed coordinates: the Gaussian (the prior box is far from it)
    assert np.all(np.abs(flat[:, 3:].mean(axis=0) - base.c[2:]) < 0.1 * base.s[2:])
    assert np.all(np.abs(flat[:, 3:].std(axis=0) / base.s[2:] - 1) < 0.1)
    # (v1, v2): the Gaussian times the prior volume along the symmetry axis,
    # Z(v1, v2) = integral of exp(v0) over the allowed interval, on a grid
    g1 = base.c[0] + base.s[0] * np.linspace(-6, 6, 241)
    g2 = base.c[1] + base.s[1] * np.linspace(-6, 6, 241)
    V1, V2 = np.meshgrid(g1, g2, indexing="ij")
    lo = np.maximum.reduce([np.full_like(V1, np.log(0.01)), np.log(2e-4) - V2, V1 - np.log(500.0)])
    hi = np.minimum.reduce([np.full_like(V1, np.log(0.2)), np.log(2.5e-3) - V2, V1 - np.log(100.0)])
    w = np.exp(-0.5 * (((V1 - base.c[0]) / base.s[0]) ** 2 + ((V2 - base.c[1]) / base.s[1]) ** 2))
    w *= np.clip(np.exp(hi) - np.exp(lo), 0, None)
    w /= w.sum()
    m1, m2 = (w * V1).sum(), (w * V2).sum()
    s1 = np.sqrt((w * (V1 - m1) ** 2).sum())
    s2 = np.sqrt((w * (V2 - m2) ** 2).sum())
    assert abs(flat[:, 1].mean() - m1) < 0.1 * s1 and abs(flat[:, 2].mean() - m2) < 0.1 * s2
    assert abs(flat[:, 1].std() / s1 - 1) < 0.1 and abs(flat[:, 2].std() / s2 - 1) < 0.1
    # the symmetry axis: given the rest, exp(v0) on the allowed interval; its
    # mean matches the mean of exact prior-conditional redraws of the same rows
    ref = lc.prior.redraw_axis(flat[::7], 0, rng)[:, 0]
    assert abs(flat[:, 0].mean() - ref.mean()) < 0.05 * flat[:, 0].std() + 0.01
    assert np.all(mcmc.rhat(v) < 1.05)
    assert r.history["stage2_accept"] > 0.3


class CorrelatedStub(GaussianStub):
    """Gaussian posterior with strong correlations (Dw-rho-T), as the front
    position 2 sqrt(Dw rho) T makes them in the tumour model."""

    def __init__(self):
        super().__init__()
        rng = np.random.default_rng(7)
        Q, _ = np.linalg.qr(rng.standard_normal((6, 6)))
        ev = np.array([1.0, 0.5, 0.2, 0.05, 0.01, 0.002])
        C = Q @ np.diag(ev) @ Q.T
        self.cov = C * np.outer(self.sd, self.sd)
        self.prec = np.linalg.inv(self.cov)

    def loglik(self, th, with_grad):
        th = np.atleast_2d(th)
        self.solves += th.shape[0]
        r = th - self.mu
        lp = self.prior.logp(th)
        return -0.5 * np.einsum("ij,jk,ik->i", r, self.prec, r) + lp, -r @ self.prec


def test_find_mode_hessian_and_preconditioned_samplers():
    rng = np.random.default_rng(5)
    post = CorrelatedStub()
    starts = post.mu + 3 * post.sd * rng.standard_normal((3, 6))
    th, lp, cov, hist = mcmc.find_mode(post, starts, iters=6)
    assert np.all(np.abs(th - post.mu) < 1e-6 * post.sd)
    # the Gaussian approximation adds the prior box's precision 12 / width^2
    w = post.prior.width
    expect = np.linalg.inv(post.prec + np.diag(12.0 / w ** 2))
    assert np.allclose(cov, expect, rtol=1e-5, atol=1e-8 * np.abs(expect).max())
    assert hist[-1] >= hist[0]
    L = np.linalg.cholesky(cov)
    th0 = th + rng.standard_normal((16, 6)) @ L.T
    r = mcmc.mala(post, th0, 800, 1.0, rng, burn=200, chol=L)
    s = r.samples[200:].reshape(-1, 6)
    assert 0.4 < r.accept < 0.75
    assert np.all(np.abs(s.mean(axis=0) - post.mu) < 0.15 * post.sd)
    assert np.all(np.abs(np.sqrt(np.diag(np.cov(s, rowvar=False))) / np.sqrt(np.diag(post.cov)) - 1) < 0.15)
    r2 = mcmc.rwm(post, th0, 2000, 1.0, rng, burn=400, chol=L)
    assert 0.15 < r2.accept < 0.35
    # preconditioning makes the ill-conditioned target easy: ESS per step
    # is far above that of the width-scaled random walk
    r3 = mcmc.rwm(post, th0, 2000, 1e-3, rng, burn=400)
    assert mcmc.ess(r2.samples[400:]).min() > 5 * mcmc.ess(r3.samples[400:]).min()


def test_log_coordinates_density_gradient_and_prior():
    post = GaussianStub()
    post.prior = mcmc.Prior(lo=0.5 * post.mu, hi=1.5 * post.mu, seed_mask=post.prior.seed_mask)
    lc = mcmc.LogCoords(post)
    th = post.mu + 0.3 * post.sd
    u = lc.to_u(th)
    assert np.allclose(lc.to_theta(u), th)
    l, g = lc.loglik(u[None], True)
    l0, g0 = post.loglik(th[None], True)
    assert np.isclose(l[0], l0[0] + np.log(th[[0, 1, 5]]).sum())
    # gradient in u against central differences of the u-density
    for i in range(6):
        e = np.zeros(6)
        e[i] = 1e-6 * max(1.0, abs(u[i]))
        fd = (lc.loglik((u + e)[None], False)[0][0] - lc.loglik((u - e)[None], False)[0][0]) / (2 * e[i])
        assert abs(fd - g[0, i]) <= 1e-5 * max(1.0, abs(fd))
    # the prior box maps to a box in u; outside it the density is -inf
    assert np.allclose(lc.prior.lo[[0, 1, 5]], np.log(post.prior.lo[[0, 1, 5]]))
    out = u.copy()
    out[0] = lc.prior.hi[0] + 0.1
    assert lc.prior.logp(out[None])[0] == -np.inf and np.isfinite(lc.prior.logp(u[None])[0])


def test_within_chain_ess_gives_no_credit_for_spread_starts():
    # stuck chains started at independent points: the multi-chain ESS counts
    # the starting spread (about m/2), the within-chain ESS does not
    rng = np.random.default_rng(2)
    x = np.repeat(rng.standard_normal((1, 64, 1)), 500, axis=0) + 1e-3 * rng.standard_normal((500, 64, 1))
    assert mcmc.ess(x)[0] > 20
    assert mcmc.ess(x, within=True)[0] > 1e4  # white noise within each chain
    # AR(1) chains started in stationarity: both agree
    phi = 0.8
    y = np.zeros((4000, 8, 1))
    y[0] = rng.standard_normal((8, 1)) / np.sqrt(1 - phi ** 2)
    for t in range(1, y.shape[0]):
        y[t] = phi * y[t - 1] + rng.standard_normal((8, 1))
    a, b = mcmc.ess(y)[0], mcmc.ess(y, within=True)[0]
    assert abs(a - b) < 0.15 * a


def test_refine_cov_recovers_a_wider_direction():
    """Laplace covariance too narrow along one direction: the profile fit
    restores the true standard deviation."""
    post = CorrelatedStub()
    wrong = post.cov.copy()
    ev, V = np.linalg.eigh(np.linalg.inv(post.cov / np.outer(post.prior.width, post.prior.width)))
    # shrink the softest direction's variance 4x
    ev2 = ev.copy()
    ev2[0] *= 16.0
    w = post.prior.width
    wrong = np.linalg.inv((V * ev2) @ V.T) * np.outer(w, w)
    cov, ratio = mcmc.refine_cov(post, post.mu, wrong)
    r = np.sort(ratio)
    assert abs(r[-1] - 4.0) < 0.05 and np.all(np.abs(r[:-1] - 1.0) < 0.05)
    assert np.allclose(cov, post.cov, rtol=1e-2, atol=1e-3 * np.abs(post.cov).max())


def test_refine_cov_reports_a_higher_profile_point():
    """Centre short of the mode along the soft direction of a correlated
    Gaussian (as damped Newton can stop part way along a narrow ridge): the
    profiles return a point above the centre, closer to the mode; at the
    mode none is higher."""
    post = CorrelatedStub()
    w = post.prior.width
    A = np.linalg.inv(post.cov / np.outer(w, w))
    ev, V = np.linalg.eigh(A)
    soft = V[:, 0] * w / np.sqrt(ev[0])   # one sd along the softest direction
    start = post.mu + 5.0 * soft
    l0 = post.loglik(start[None], False)[0][0]
    _, _, best, lb = mcmc.refine_cov(post, start, post.cov, with_best=True)
    assert lb > l0 + 1.0
    z = lambda u: (u - post.mu) / w
    assert np.linalg.norm(z(best)) < 0.5 * np.linalg.norm(z(start))
    lm = post.loglik(post.mu[None], False)[0][0]
    _, _, _, lbm = mcmc.refine_cov(post, post.mu, post.cov, with_best=True)
    assert lbm <= lm + 1e-9


class BananaStub(GaussianStub):
    """A narrow curved ridge in coordinates z = (theta - mu) / sd (the prior
    box is |z| <= 20):
    log pi = -(z0^2 + ((z1 - k z0^2) / eps)^2 + z2^2 + ... + z5^2) / 2,
    mode at mu; its conditional width across the ridge is eps."""

    def __init__(self, k=0.1, eps=0.02):
        super().__init__()
        self.k, self.eps = k, eps

    def _z(self, th):
        return (np.atleast_2d(th) - self.mu) / self.sd

    def loglik(self, th, with_grad):
        th = np.atleast_2d(th)
        self.solves += th.shape[0]
        z = self._z(th)
        r = (z[:, 1] - self.k * z[:, 0] ** 2) / self.eps
        lp = -0.5 * (z[:, 0] ** 2 + r ** 2 + np.sum(z[:, 2:] ** 2, axis=1))
        gz = np.zeros_like(z)
        gz[:, 0] = -z[:, 0] + r / self.eps * 2 * self.k * z[:, 0]
        gz[:, 1] = -r / self.eps
        gz[:, 2:] = -z[:, 2:]
        return lp + self.prior.logp(th), gz / self.sd


def test_polish_mode_reaches_the_mode_along_a_curved_ridge():
    """Newton started far along the ridge (across-ridge width 1/50 of the
    along-ridge one, as in the tumour model's (log rho T, log Dw/rho)) and cut
    short stops below the mode; polish_mode restarts it from higher profile
    points until no profile point is higher, and ends at the mode."""
    post = BananaStub()
    w = post.sd
    z0 = np.zeros(6)
    z0[0], z0[1] = 5.0, post.k * 25.0  # on the ridge, 12.5 nats below the mode
    start = post.mu + z0 * w
    v, lp, cov0, _ = mcmc.find_mode(post, start[None], iters=1)
    lm = post.loglik(post.mu[None], False)[0][0]
    assert lp < lm - 1.0  # one Newton step does not get there
    v2, lp2, _, cov, restarts = mcmc.polish_mode(post, v, lp, cov0, polish=8, gain=0.01)
    assert restarts >= 1
    assert lp2 > lm - 0.05
    assert np.all(np.abs((v2 - post.mu) / w) < 0.2)
    assert np.all(np.isfinite(cov)) and np.all(np.linalg.eigvalsh(cov) > 0)


def test_stranded_chains_and_discrepancy():
    lp = np.array([0.0, -1.0, -2.0, -3.0, -40.0, -np.inf])
    assert mcmc._stranded(lp).tolist() == [False, False, False, False, True, True]
    assert mcmc._stranded(np.full(3, -np.inf)).all()
    # a constant offset between exact and surrogate costs nothing
    assert mcmc._discrepancy(lp[:4], lp[:4] - 7.0) == 0.0
    assert mcmc._discrepancy(lp[:2], lp[:2]) == np.inf  # too few finite pairs


def test_invariant_coordinates_map_gradient_and_symmetry():
    post = GaussianStub()
    post.prior = mcmc.Prior(lo=0.5 * post.mu, hi=1.5 * post.mu, seed_mask=post.prior.seed_mask)
    lc = mcmc.LogCoords(post, A=mcmc.INVARIANT_MAP)
    th = post.mu * (1 + 0.05 * np.arange(6) / 6)
    v = lc.to_u(th)
    assert np.allclose(lc.to_theta(v), th)
    # the scaling (c Dw, c rho, T / c) moves v_0 only
    c = 1.07
    th2 = th.copy()
    th2[0] *= c
    th2[1] *= c
    th2[5] /= c
    dv = lc.to_u(th2) - v
    assert abs(dv[0] - np.log(c)) < 1e-12 and np.all(np.abs(dv[1:]) < 1e-12)
    l, g = lc.loglik(v[None], True)
    for i in range(6):
        e = np.zeros(6)
        e[i] = 1e-6
        fd = (lc.loglik((v + e)[None], False)[0][0] - lc.loglik((v - e)[None], False)[0][0]) / 2e-6
        assert abs(fd - g[0, i]) <= 1e-4 * max(1.0, abs(fd)), (i, fd, g[0, i])
    # prior: inside the box finite, the image box bounds contain the point
    assert np.isfinite(lc.prior.logp(v[None])[0])
    assert np.all(lc.prior.lo <= v) and np.all(v <= lc.prior.hi)


class FieldModelStub:
    """Posterior-like object whose 'solver' returns fields of a known
    second-order model phi(u) = f0 + sum_i a_i u_i + b u_0^2 / 2 + sum_i c_i u_0 u_i
    (no clamping), and a handle whose affine model is evaluated in NumPy."""

    def __init__(self, n_cells=50, seed=0):
        rng = np.random.default_rng(seed)
        self.f0 = rng.uniform(0.3, 0.6, n_cells)
        self.a = rng.normal(0, 0.1, (6, n_cells))
        self.b = rng.normal(0, 0.2, n_cells)
        self.c = rng.normal(0, 0.1, (6, n_cells))
        self.c[0] = 0.0
        self.target = self.field(np.full(6, 0.01)) + 0.001 * rng.standard_normal(n_cells)
        self.prior = mcmc.Prior(lo=np.full(6, -1.0), hi=np.full(6, 1.0),
                                seed_mask=np.ones((4, 4, 4), dtype=bool))
        self.prior.logp = lambda th: np.zeros(np.atleast_2d(th).shape[0])
        self.handle, self.L, self.dt0, self.ic_peak, self.ic_sigma = self, 1.0, 1.0, 0.1, 1.0
        self.max_samples = 7

    def field(self, u):
        return (self.f0 + u @ self.a + 0.5 * self.b * u[0] ** 2 + u[0] * (u @ self.c))

    def loglik_exact(self, u):
        return -0.5 * np.sum((self.field(u) - self.target) ** 2) / 1e-4

    def batch_solve(self, rows, L, ic_peak, ic_sigma, with_loglik, want_phi, dt0):
        return {"phi": np.array([self.field(np.array(r)) for r in rows])}

    def affine_set(self, phi0, J):
        self._phi0, self._J = phi0.astype(np.float64), J.astype(np.float64)

    def affine_loglik(self, coeffs):
        f = self._phi0[None] + coeffs @ self._J
        return -0.5 * np.sum((f - self.target) ** 2, axis=1) / 1e-4


def test_tangent_surrogate_second_order_terms_along_the_axis():
    m = FieldModelStub()
    ref = np.zeros(6)
    rng = np.random.default_rng(4)
    us = 0.2 * rng.standard_normal((20, 6))
    exact = np.array([m.loglik_exact(u) for u in us])
    # a handle holds one affine model: the latest build is the active one
    lin = mcmc.AffineSurrogate(m, ref, np.full(6, 0.05))
    err_lin = np.abs(lin.logpost(us) - exact).max()
    quad = mcmc.AffineSurrogate(m, ref, np.full(6, 0.05), quad_axis=0)
    assert np.allclose(quad.logpost(us), exact, rtol=1e-6, atol=1e-6 * np.abs(exact).max())
    assert err_lin > 100 * np.abs(quad.logpost(us) - exact).max()
    assert quad.J.shape == (12, m.f0.size)


def test_redraw_axis_samples_the_prior_conditional():
    """Along the scaling symmetry (v_0 of the invariant coordinates) the
    prior conditional is exp(v_0) on the interval the box allows; the redraw
    reproduces it (Kolmogorov distance of 20000 draws) and stays in the box."""
    post = GaussianStub()
    post.prior = mcmc.Prior(lo=np.array([2e-4, 0.01, 0, 0, 0, 100.0]),
                            hi=np.array([2.5e-3, 0.2, 64, 64, 64, 500.0]),
                            seed_mask=np.ones((64, 64, 64), dtype=bool))
    lc = mcmc.LogCoords(post, A=mcmc.INVARIANT_MAP)
    v = lc.to_u(np.array([6e-4, 0.15, 30.0, 32.0, 31.0, 260.0]))
    rng = np.random.default_rng(0)
    draws = lc.prior.redraw_axis(np.repeat(v[None], 20000, axis=0), 0, rng)
    assert np.all(draws[:, 1:] == v[1:])
    assert np.all(np.isfinite(lc.prior.logp(draws)))
    # interval: log rho in [log .01, log .2], log Dw = v2 + v0 in box, log T = v1 - v0 in box
    lo = max(np.log(0.01), np.log(2e-4) - v[2], v[1] - np.log(500.0))
    hi = min(np.log(0.2), np.log(2.5e-3) - v[2], v[1] - np.log(100.0))
    x = np.sort(draws[:, 0])
    cdf = (np.exp(x) - np.exp(lo)) / (np.exp(hi) - np.exp(lo))
    emp = np.arange(1, x.size + 1) / x.size
    assert x[0] >= lo - 1e-12 and x[-1] <= hi + 1e-12
    assert np.abs(cdf - emp).max() < 0.015


def _invariant_moments(base):
    """Posterior moments of (v1, v2) for InvariantStub: the Gaussian times the
    prior volume along the symmetry axis, on a grid."""
    g1 = base.c[0] + base.s[0] * np.linspace(-6, 6, 241)
    g2 = base.c[1] + base.s[1] * np.linspace(-6, 6, 241)
    V1, V2 = np.meshgrid(g1, g2, indexing="ij")
    lo = np.maximum.reduce([np.full_like(V1, np.log(0.01)), np.log(2e-4) - V2, V1 - np.log(500.0)])
    hi = np.minimum.reduce([np.full_like(V1, np.log(0.2)), np.log(2.5e-3) - V2, V1 - np.log(100.0)])
    w = np.exp(-0.5 * (((V1 - base.c[0]) / base.s[0]) ** 2 + ((V2 - base.c[1]) / base.s[1]) ** 2))
    w *= np.clip(np.exp(hi) - np.exp(lo), 0, None)
    w /= w.sum()
    m1, m2 = (w * V1).sum(), (w * V2).sum()
    return m1, m2, np.sqrt((w * (V1 - m1) ** 2).sum()), np.sqrt((w * (V2 - m2) ** 2).sum())


def test_axis_log_marginal_integrates_the_prior_along_the_axis():
    base = InvariantStub()
    lc = mcmc.LogCoords(base, A=mcmc.INVARIANT_MAP)
    rng = np.random.default_rng(4)
    th = np.column_stack([rng.uniform(3e-4, 2e-3, 6), rng.uniform(0.02, 0.18, 6),
                          rng.uniform(22, 42, (6, 3)), rng.uniform(120, 480, 6)])
    v = lc.to_u(th)
    got = lc.prior.axis_log_marginal(v, 0)
    ts = np.linspace(-8, 8, 400001)
    for r in range(len(v)):
        pts = np.repeat(v[r:r + 1], ts.size, axis=0)
        pts[:, 0] += ts
        lp = lc.prior.logp(pts)
        mx = lp[np.isfinite(lp)].max()
        ref = np.log(np.trapezoid(np.exp(lp - mx), ts)) + mx
        assert abs(got[r] - ref) < 1e-4, (r, got[r], ref)
    far = v[:1].copy()
    far[0, 2] = 10.0  # log Dw/rho far outside what the box allows
    assert np.isneginf(lc.prior.axis_log_marginal(far, 0)[0])


def test_plain_chains_sample_the_invariant_posterior():
    """The plain single-solve sampler (Laplace-preconditioned random walk on
    the identified coordinates, the symmetry axis redrawn from its prior
    conditional and the prior marginal in the ratio): one solve per step and
    the exact posterior's moments."""
    rng = np.random.default_rng(9)
    base = InvariantStub()
    lc = mcmc.LogCoords(base, A=mcmc.INVARIANT_MAP)
    v_c = np.concatenate([[np.log(0.15)], base.c])
    v0 = v_c + np.concatenate([[0.0], 2 * base.s]) * rng.standard_normal((4, 6))
    v0 = lc.prior.redraw_axis(v0, 0, rng)
    cov = np.diag(np.concatenate([[0.3], base.s]) ** 2)
    steps, burn = 6000, 500
    s0 = base.solves
    r = mcmc.plain_chains(lc, v0, steps, cov, rng, burn=burn)
    assert base.solves - s0 <= 4 * (steps + 1)
    v = r.samples[burn:]
    flat = v.reshape(-1, 6)
    assert np.all(np.abs(flat[:, 3:].mean(axis=0) - base.c[2:]) < 0.1 * base.s[2:])
    assert np.all(np.abs(flat[:, 3:].std(axis=0) / base.s[2:] - 1) < 0.1)
    m1, m2, s1, s2 = _invariant_moments(base)
    assert abs(flat[:, 1].mean() - m1) < 0.1 * s1 and abs(flat[:, 2].mean() - m2) < 0.1 * s2
    assert abs(flat[:, 1].std() / s1 - 1) < 0.1 and abs(flat[:, 2].std() / s2 - 1) < 0.1
    ref = lc.prior.redraw_axis(flat[::7], 0, rng)[:, 0]
    assert abs(flat[:, 0].mean() - ref.mean()) < 0.05 * flat[:, 0].std() + 0.01
    assert np.all(mcmc.rhat(v) < 1.05)
    assert 0.15 < r.accept < 0.4


def test_tmcmc_recovers_a_gaussian_and_its_evidence():
    """TMCMC from prior draws on the Gaussian stub inside its prior box:
    the final population's moments and the log evidence
    log( integral of exp(-z^2/2) / box volume ) = sum log(sqrt(2 pi) sd / width)."""
    rng = np.random.default_rng(3)
    post = GaussianStub()
    th0 = post.prior.lo + post.prior.width * rng.random((4000, 6))
    r = mcmc.tmcmc(post, th0, rng)
    assert r.p[0] == 0.0 and r.p[-1] == 1.0 and np.all(np.diff(r.p) > 0)
    assert len(r.p) > 3
    s = r.theta
    assert s.shape == (4000, 6)
    assert np.all(np.abs(s.mean(axis=0) - post.mu) < 0.1 * post.sd)
    assert np.all(np.abs(s.std(axis=0) / post.sd - 1) < 0.15)
    exact = float(np.sum(np.log(np.sqrt(2 * np.pi) * post.sd / post.prior.width)))
    assert abs(r.log_evidence - exact) < 0.25, (r.log_evidence, exact)
    assert r.solves >= 4000 * len(r.p)
    assert all(0.1 < a < 0.6 for a in r.accept[2:])
    # Ching & Chen's original: chains as long as a leader's multiplicity,
    # fixed beta^2 = 0.04 (its moments only: its evidence is biased low)
    r0 = mcmc.tmcmc(post, th0, rng, max_chain=0, steps_per_state=1, target_accept=None)
    assert r0.p[-1] == 1.0
    assert np.all(np.abs(r0.theta.mean(axis=0) - post.mu) < 0.5 * post.sd)
    assert np.all(np.abs(r0.theta.std(axis=0) / post.sd - 1) < 0.2)


def test_tmcmc_on_the_invariant_posterior_in_log_coordinates():
    """TMCMC in the scaling symmetry's coordinates (prior density with its
    Jacobian; the likelihood flat along v0) from prior draws: the identified
    coordinates' moments."""
    rng = np.random.default_rng(5)
    base = InvariantStub()
    lc = mcmc.LogCoords(base, A=mcmc.INVARIANT_MAP)
    lo, hi = base.prior.lo, base.prior.hi
    v0 = lc.to_u(lo + (hi - lo) * rng.random((3000, 6)))
    r = mcmc.tmcmc(lc, v0, rng)
    assert r.p[-1] == 1.0 and len(r.p) > 5
    m1, m2, s1, s2 = _invariant_moments(base)
    f = r.theta
    assert abs(f[:, 1].mean() - m1) < 0.15 * s1 and abs(f[:, 2].mean() - m2) < 0.15 * s2
    assert abs(f[:, 1].std() / s1 - 1) < 0.2 and abs(f[:, 2].std() / s2 - 1) < 0.2
    assert np.all(np.abs(f[:, 3:].mean(axis=0) - base.c[2:]) < 0.15 * base.s[2:])


def test_delayed_acceptance_with_independence_moves_targets_the_posterior():
    """The inner chain with independence proposals (a Gaussian fitted to the
    population in burn-in, inflated) next to the random walk and the axis
    redraws: delayed acceptance still samples the invariant stub's
    posterior (same checks as the axis-redraw test)."""
    rng = np.random.default_rng(12)
    base = InvariantStub()
    lc = mcmc.LogCoords(base, A=mcmc.INVARIANT_MAP)
    sp = lc.surrogate(mcmc.SurrogatePosterior(InvariantSurrogate(base), base.prior))
    v_c = np.concatenate([[np.log(0.15)], base.c])
    v0 = v_c + np.concatenate([[0.0], base.s]) * rng.standard_normal((32, 6))
    v0 = lc.prior.redraw_axis(v0, 0, rng)
    chol = np.diag(np.concatenate([[0.1], base.s]))
    r = mcmc.da(lc, sp, v0, 1500, 1.0, rng, inner=6, burn=300, chol=chol, adapt=True, axis=0,
                axis_prob=0.3, ind_prob=0.4)
    v = r.samples[300:]
    flat = v.reshape(-1, 6)
    assert np.all(np.abs(flat[:, 3:].mean(axis=0) - base.c[2:]) < 0.1 * base.s[2:])
    assert np.all(np.abs(flat[:, 3:].std(axis=0) / base.s[2:] - 1) < 0.1)
    m1, m2, s1, s2 = _invariant_moments(base)
    assert abs(flat[:, 1].mean() - m1) < 0.1 * s1 and abs(flat[:, 2].mean() - m2) < 0.1 * s2
    assert abs(flat[:, 1].std() / s1 - 1) < 0.1 and abs(flat[:, 2].std() / s2 - 1) < 0.1
    assert np.all(mcmc.rhat(v) < 1.05)


def test_inner_chain_independence_moves_sample_the_screen():
    """inner_chain's independence move alone (probability 1, a deliberately
    wrong Gaussian) samples the screen's density: long chains of a 1-D-like
    Gaussian screen reach its mean and spread."""
    rng = np.random.default_rng(13)

    class Screen:
        def logpost(self, v):
            v = np.atleast_2d(v)
            return -0.5 * np.sum(((v - 1.0) / 0.5) ** 2, axis=1)

    class Flat:
        def logp(self, v):
            return np.zeros(np.atleast_2d(v).shape[0])

    y0 = np.zeros((400, 6))
    sc = Screen()
    G = np.diag(np.full(6, 0.8))
    y, ly, na, nt = mcmc.inner_chain(Flat(), sc, y0, sc.logpost(y0), 60, 0.5, np.eye(6), None, 0.0, rng,
                                     ind=(1.0, np.full(6, 0.7), G))
    assert nt == 0  # every step was an independence move
    assert np.all(np.abs(y.mean(axis=0) - 1.0) < 0.1)
    assert np.all(np.abs(y.std(axis=0) / 0.5 - 1) < 0.15)
