"""GPU: the affine (tangent) density model and the batched + adjoint +
surrogate posterior pipeline.

* gbg_affine_loglik at delta = 0 is the batched solver's log L of the
  reference sample, bit for bit (same field, same likelihood kernel);
* at other deltas it is the likelihood of phi0 + J delta, clamped and masked,
  as a NumPy restatement fed through gbg_set_phi + gbg_loglik computes it;
* the pipeline (prior screen, adjoint Newton mode, profile-refined Gaussian,
  delayed acceptance with the affine screen) runs on a small problem with
  working acceptance rates, draws inside the prior, and two halves of the
  chain population agreeing on the posterior mean within half a posterior
  standard deviation.
"""
import numpy as np
import pytest

from gliomauq_gb300 import _lib, mcmc, synthetic as S

pytestmark = pytest.mark.gpu
LIK = (0.0025, 1.0, 0.7, 0.25, 0.09)
N = 32


def _problem(h, an):
    truth = S.SampleParams(Dw=0.0013, rho=0.08, x0=15.2, y0=16.1, z0=15.7, T=150.0)
    u = h.batch_solve([truth.as_tuple()], an.L, with_loglik=False, want_phi=True)["phi"][0]
    obs = S.make_observations(u.astype(np.float64), an, seed=3, centre_xyz=(15, 16, 15),
                              radius_vox=9.0)
    h.set_observations(obs.pet, obs.t1, obs.t2, obs.points, LIK)
    return truth


def test_affine_model_matches_solver_and_restatement(gbg):
    an = S.make_anatomy(N, seed=4)
    with _lib.Handle(N, "f32", max_samples=16) as h:
        h.set_anatomy(an.p_w, an.p_g)
        truth = _problem(h, an)
        dt0 = S.reference_dt(N, 0.0025, an.L)[0]
        r = h.batch_solve([truth.as_tuple()], an.L, want_phi=True, dt0=dt0)
        phi0 = r["phi"][0]
        rng = np.random.default_rng(1)
        J = (rng.standard_normal((6, N, N, N)) * 0.05 * (phi0 > 0)).astype(np.float32)
        h.affine_set(phi0, J)
        l0 = h.affine_loglik(np.zeros((1, 6)))
        assert l0[0] == r["loglik"][0]["total"]
        deltas = rng.standard_normal((5, 6))
        got = h.affine_loglik(deltas)
        msk = np.zeros(N ** 3, dtype=bool)
        # the fast path's mask: tissue cells whose six face neighbours are tissue
        b = (an.p_w + an.p_g) > 0
        m = b.copy()
        for ax in range(3):
            m &= np.roll(b, 1, axis=ax) & np.roll(b, -1, axis=ax)
        for i, d in enumerate(deltas):
            f = phi0.astype(np.float64) + np.tensordot(d, J.astype(np.float64), axes=1)
            f = np.where(m, np.clip(f, 0.0, 1.0), 0.0)
            h.set_phi(f)
            ref = h.loglik()["total"]
            assert abs(got[i] - ref) <= 1e-5 * abs(ref), (i, got[i], ref)


def test_posterior_pipeline_small(gbg):
    an = S.make_anatomy(N, seed=4)
    with _lib.Handle(N, "f32", max_samples=64) as h:
        h.set_anatomy(an.p_w, an.p_g)
        _problem(h, an)
        prior = mcmc.Prior.from_anatomy(an)
        dt0 = S.reference_dt(N, prior.hi[0], an.L)[0]
        screen = np.array([p.as_tuple() for p in S.draw_prior(an, 128, seed=9)])
        rng = np.random.default_rng(0)
        res = mcmc.sample_posterior(h, an.L, prior, dt0, rng, chains=32, generations=120,
                                    burn=40, inner=8, screen_draws=screen)
        th = res.theta
        hist = res.result.history
        print("stage1", hist["stage1_accept"], "stage2", hist["stage2_accept"],
              "ess", mcmc.ess(th, within=True))
        assert np.isfinite(th).all() and np.all(np.isfinite(prior.logp(th.reshape(-1, 6))))
        assert 0.1 < hist["stage1_accept"] < 0.6
        assert hist["stage2_accept"] > 0.3
        # two independent halves of the population agree on the posterior
        # mean: with a few hundred effective draws per half the standard error
        # of each half's mean is below 0.1 posterior sd
        a = th[:, :16].reshape(-1, 6).mean(axis=0)
        b = th[:, 16:].reshape(-1, 6).mean(axis=0)
        sd = th.reshape(-1, 6).std(axis=0)
        assert np.all(np.abs(a - b) <= 0.5 * sd), (a, b, sd)


def _screen(h, an, prior):
    """The tangent screen of the small problem around its mode, in the
    invariant coordinates, and the refined Laplace covariance."""
    dt0 = S.reference_dt(N, prior.hi[0], an.L)[0]
    lc = mcmc.LogCoords(mcmc.Posterior(h, an.L, dt0, prior), A=mcmc.INVARIANT_MAP)
    screen = np.array([p.as_tuple() for p in S.draw_prior(an, 128, seed=9)])
    dv = lc.to_u(screen)
    ld, _ = lc.loglik(dv, False)
    v_map, lp_map, cov0, _ = mcmc.find_mode(lc, dv[np.argsort(ld)[::-1][:4]], iters=10)
    v_map, lp_map, cov0, cov, _ = mcmc.polish_mode(lc, v_map, lp_map, cov0)
    sur = mcmc.AffineSurrogate(lc, v_map, 0.5 * np.sqrt(np.diag(cov)), quad_axis=0)
    return lc, sur, v_map, cov


def test_gpu_screening_chain_evaluates_the_screen_density(gbg):
    """gbg_affine_chain with 0 steps returns log pi* = the affine model's log L
    (gbg_affine_loglik) + the prior in the sampler's coordinates, to the
    last bits of the reduction order (1e-12 relative), -inf outside."""
    an = S.make_anatomy(N, seed=4)
    with _lib.Handle(N, "f32", max_samples=64) as h:
        h.set_anatomy(an.p_w, an.p_g)
        _problem(h, an)
        prior = mcmc.Prior.from_anatomy(an)
        lc, sur, v_map, cov = _screen(h, an, prior)
        rng = np.random.default_rng(4)
        v = v_map + 3.0 * rng.standard_normal((40, 6)) @ np.linalg.cholesky(cov).T
        v[:3, 1] += 50.0  # far outside the prior
        exp = sur.logpost(v)
        y, l0, l1, a1 = sur.chain(v, 0, 0.1, np.eye(6), 0, 0.5, 1)
    assert np.array_equal(y, v)
    fin = np.isfinite(exp)
    assert np.array_equal(fin, np.isfinite(l0)) and np.array_equal(l0, l1)
    assert not fin[:3].any() and fin[3:].sum() > 10
    assert np.all(np.abs(l0[fin] - exp[fin]) <= 1e-12 * np.abs(exp[fin]))


def test_gpu_screening_chain_samples_the_screen_density(gbg):
    """The GPU inner chain's invariant law is the screen's posterior pi*:
    the moments of the identified coordinates after 256 chains x 400 steps
    equal those of importance sampling pi* (evaluated by
    gbg_affine_loglik) from a widened Laplace Gaussian, within 0.1 sd, and
    the acceptance of its random-walk moves is in range."""
    an = S.make_anatomy(N, seed=4)
    with _lib.Handle(N, "f32", max_samples=256) as h:
        h.set_anatomy(an.p_w, an.p_g)
        _problem(h, an)
        prior = mcmc.Prior.from_anatomy(an)
        lc, sur, v_map, cov = _screen(h, an, prior)
        Lc = np.linalg.cholesky(mcmc._decoupled(cov, 0))
        rng = np.random.default_rng(5)
        v0 = lc.prior.redraw_axis(v_map + rng.standard_normal((256, 6)) @ Lc.T, 0, rng)
        v0[~np.isfinite(lc.prior.logp(v0))] = v_map
        y, _, _, a1 = sur.chain(v0, 100, 2.38 / np.sqrt(5), Lc, 0, 0.5, 7)  # burn-in
        draws = []
        for k in range(6):
            y, _, _, a1 = sur.chain(y, 50, 2.38 / np.sqrt(5), Lc, 0, 0.5, 100 + k)
            draws.append(y.copy())
        draws = np.concatenate(draws)
        # importance sampling of pi* on the identified coordinates
        q_cov = 2.25 * cov
        Lq = np.linalg.cholesky(q_cov)
        x = v_map + rng.standard_normal((20000, 6)) @ Lq.T
        x = lc.prior.redraw_axis(x, 0, rng)  # the axis from its prior conditional
        # q density of the identified part times the prior conditional of the
        # axis: pi*(x) / q(x) = L*(x) m(x_id) / N(x_id)
        lq_id = -0.5 * np.sum(np.linalg.solve(np.linalg.cholesky(q_cov[1:, 1:]),
                                              (x[:, 1:] - v_map[1:]).T) ** 2, axis=0)
        lstar = sur.logpost(x) - lc.prior.logp(x)
        lw = lstar + lc.prior.axis_log_marginal(x, 0) - lq_id
        lw = np.where(np.isfinite(lw), lw, -np.inf)
        w = np.exp(lw - lw.max())
        w /= w.sum()
    print("random-walk acceptance", a1, "IS ess", 1.0 / np.sum(w ** 2))
    assert 0.1 < a1 < 0.6
    assert 1.0 / np.sum(w ** 2) > 500
    m_is = w @ x[:, 1:]
    sd_is = np.sqrt(w @ (x[:, 1:] - m_is) ** 2)
    m_ch = draws[:, 1:].mean(axis=0)
    sd_ch = draws[:, 1:].std(axis=0)
    print("mean diff / sd", (m_ch - m_is) / sd_is, "sd ratio", sd_ch / sd_is)
    assert np.all(np.abs(m_ch - m_is) < 0.1 * sd_is)
    assert np.all(np.abs(sd_ch / sd_is - 1) < 0.1)
