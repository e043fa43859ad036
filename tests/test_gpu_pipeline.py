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
    """gbg_affine_chain with 0 steps returns its screen density log pi*: the
    affine model's log L + the prior in the sampler's coordinates, with the
    per-point terms in float (within 1e-6 relative + 1e-3 of the double
    evaluation by gbg_affine_loglik), -inf outside the prior."""
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
    err = np.abs(l0[fin] - exp[fin])
    print("float screen vs double: max abs", err.max(), "max rel", (err / np.abs(exp[fin])).max())
    assert np.all(err <= 1e-6 * np.abs(exp[fin]) + 1e-3)


@pytest.mark.parametrize("with_ind", [False, True])
def test_gpu_screening_chain_moves_like_the_host_chain(gbg, with_ind):
    """The GPU inner chain is the host inner chain (mcmc.inner_chain) with
    other random numbers: from the same 1024 starting points, after 60
    steps, the two populations agree in mean (within 5 standard errors of
    the difference) and spread (10 %), and in random-walk acceptance; with
    independence moves too (from a deliberately shifted Gaussian)."""
    an = S.make_anatomy(N, seed=4)
    with _lib.Handle(N, "f32", max_samples=1024) as h:
        h.set_anatomy(an.p_w, an.p_g)
        _problem(h, an)
        prior = mcmc.Prior.from_anatomy(an)
        lc, sur, v_map, cov = _screen(h, an, prior)
        Lc = np.linalg.cholesky(mcmc._decoupled(cov, 0))
        rng = np.random.default_rng(5)
        v0 = lc.prior.redraw_axis(v_map + 1.5 * rng.standard_normal((1024, 6)) @ Lc.T, 0, rng)
        v0[~np.isfinite(lc.prior.logp(v0))] = v_map
        step = 2.38 / np.sqrt(5)
        ind = (0.3, v_map + 0.5 * Lc[:, 0] + 0.3 * np.diag(Lc), 1.3 * Lc) if with_ind else None
        ap = 0.3 if with_ind else 0.5
        yg, _, _, ag = sur.chain(v0, 60, step, Lc, 0, ap, 11, ind=ind)
        yh, _, na, nt = mcmc.inner_chain(lc.prior, sur, v0, sur.logpost(v0), 60, step, Lc, 0, ap, rng,
                                         ind=ind)
    ah = na / nt
    se = np.sqrt((yg.var(axis=0) + yh.var(axis=0)) / len(v0))
    print("acceptance gpu", ag, "host", ah, "mean diff / se", (yg.mean(axis=0) - yh.mean(axis=0)) / se,
          "sd ratio", yg.std(axis=0) / yh.std(axis=0))
    assert abs(ag - ah) < 0.03
    assert np.all(np.abs(yg.mean(axis=0) - yh.mean(axis=0)) < 5 * se)
    assert np.all(np.abs(yg.std(axis=0) / yh.std(axis=0) - 1) < 0.1)
