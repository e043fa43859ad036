"""GPU: MALA and RWM generations over the solver (smooth-time-grid log L and
adjoint gradients) on a small problem: finite densities, chains inside the
prior, acceptance rates in range, one batched call per generation."""
import numpy as np
import pytest

from gliomauq_gb300 import _lib, mcmc, synthetic as S

pytestmark = pytest.mark.gpu
LIK = (0.0025, 1.0, 0.7, 0.25, 0.09)


def test_mala_and_rwm_generations(gbg):
    an = S.make_anatomy(32, seed=4)
    truth = S.SampleParams(Dw=0.0013, rho=0.08, x0=15.2, y0=16.1, z0=15.7, T=120.0)
    rng = np.random.default_rng(0)
    with _lib.Handle(32, "f32", max_samples=1) as h:
        h.set_anatomy(an.p_w, an.p_g)
        u = h.batch_solve([truth.as_tuple()], an.L, with_loglik=False, want_phi=True)["phi"][0]
        obs = S.make_observations(u.astype(np.float64), an, seed=3, centre_xyz=(15, 16, 15),
                                  radius_vox=9.0)
        h.set_observations(obs.pet, obs.t1, obs.t2, obs.points, LIK)
        prior = mcmc.Prior.from_anatomy(an)
        post = mcmc.Posterior(h, an.L, S.reference_dt(32, prior.hi[0], an.L)[0], prior)
        th0 = np.array([truth.as_tuple()] * 4) + rng.normal(0, 1e-3, (4, 6)) * prior.width
        r = mcmc.mala(post, th0, 12, 1e-3, rng, burn=6)
        assert np.isfinite(r.samples).all() and 0.0 <= r.accept <= 1.0
        assert np.all(np.isfinite(prior.logp(r.samples.reshape(-1, 6))))
        assert post.calls == 13  # one batched call per generation (+ the start)
        r2 = mcmc.rwm(post, th0[:1], 12, 1e-3, rng, burn=6)
        assert np.isfinite(r2.samples).all()


def test_tmcmc_and_propagation_on_the_solver(gbg, oracle_lib):
    """TMCMC from prior draws over the batched solver (every Metropolis step
    of the population one batched call), then the posterior propagation
    statistics of its final population: p reaches 1, draws inside the
    prior, the population concentrated around the truth, and the mean and
    variance fields equal the oracle's statistics over the solver's own
    final densities of those samples."""
    an = S.make_anatomy(32, seed=4)
    truth = S.SampleParams(Dw=0.0013, rho=0.08, x0=15.2, y0=16.1, z0=15.7, T=120.0)
    rng = np.random.default_rng(2)
    N = 256
    with _lib.Handle(32, "f32", max_samples=N) as h:
        h.set_anatomy(an.p_w, an.p_g)
        prior = mcmc.Prior.from_anatomy(an)
        dt0 = S.reference_dt(32, prior.hi[0], an.L)[0]
        u = h.batch_solve([truth.as_tuple()], an.L, with_loglik=False, want_phi=True,
                          dt0=dt0)["phi"][0]
        obs = S.make_observations(u.astype(np.float64), an, seed=3, centre_xyz=(15, 16, 15),
                                  radius_vox=9.0)
        h.set_observations(obs.pet, obs.t1, obs.t2, obs.points, LIK)
        post = mcmc.Posterior(h, an.L, dt0, prior)
        th0 = np.array([p.as_tuple() for p in S.draw_prior(an, N, seed=11)])
        r = mcmc.tmcmc(post, th0, rng, max_stages=60)
        print("stages", len(r.p) - 1, "accept", np.round(r.accept, 2), "log Z", r.log_evidence,
              "solves", r.solves, "seconds", r.seconds)
        assert r.p[-1] == 1.0
        assert np.all(np.isfinite(prior.logp(r.theta)))
        assert np.all(np.isfinite(r.loglik))
        # the seed is identified to about a voxel
        assert np.all(np.abs(r.theta[:, 2:5].mean(axis=0) - [truth.x0, truth.y0, truth.z0]) < 1.5)
        assert r.solves >= N * (len(r.p) - 1)
        mean, var = mcmc.propagate(h, an.L, r.theta, dt0=dt0)
        phi = h.batch_solve([tuple(x) for x in r.theta], an.L, with_loglik=False, want_phi=True,
                            dt0=dt0)["phi"]
    om, ov = oracle_lib.propagation_stats(phi, reference_rules=False)
    assert np.array_equal(mean, om.astype(np.float64))
    assert np.array_equal(var, ov.astype(np.float64))
    assert mean.max() > 0.5 and var.max() > 0
