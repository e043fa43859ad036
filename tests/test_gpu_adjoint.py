"""GPU: MALA gradients from the discrete adjoint (gbg_adjoint_grad) against
central finite differences of the same forward model, h = 1e-4 relative to
each parameter; and independence from the checkpoint interval."""
import numpy as np
import pytest

from gliomauq_gb300 import _lib, synthetic as S

pytestmark = pytest.mark.gpu

LIK = (0.0025, 1.0, 0.7, 0.25, 0.09)
NAMES = ["Dw", "rho", "x0", "y0", "z0", "T"]


def _problem(n=32):
    an = S.make_anatomy(n, seed=4)
    truth = np.clip(S.gaussian_ic(an, 15.0, 16.0, 15.0, peak=0.9, sigma=2.0), 0, 1)
    obs = S.make_observations(truth, an, seed=3, centre_xyz=(15, 16, 15), radius_vox=9.0)
    samples = [(0.0013, 0.05, 15.3, 16.2, 15.6, 41.3), (0.0021, 0.12, 14.6, 15.4, 16.3, 27.7)]
    dt0 = S.reference_dt(n, 0.0025, an.L)[0]  # from the prior's largest Dw
    return an, obs, samples, dt0


def _fd(h, samples, dt0, L, state, rel=1e-4):
    g = np.zeros((len(samples), 6))
    for s, base in enumerate(samples):
        for i in range(6):
            step = rel * abs(base[i])
            p, m = list(base), list(base)
            p[i] += step
            m[i] -= step
            lp, _ = h.adjoint_grad([tuple(p)], dt0, L, state=state, want_grad=False)
            lm, _ = h.adjoint_grad([tuple(m)], dt0, L, state=state, want_grad=False)
            g[s, i] = (lp[0] - lm[0]) / (2 * step)
    return g


def _rel_err(ga, gf, samples):
    # compare relative sensitivities theta_i * dlogL/dtheta_i so the units agree
    th = np.abs(np.array(samples))
    a, f = ga * th, gf * th
    return np.linalg.norm(a - f, axis=1) / np.linalg.norm(f, axis=1), a, f


@pytest.mark.parametrize("state,tol,grid", [("f64", 1e-5, "fixed"), ("f32", 1e-3, "fixed"),
                                            ("f64", 1e-5, "scaled"), ("f32", 1e-3, "scaled")])
def test_adjoint_gradient_matches_central_differences(gbg, state, tol, grid):
    an, obs, samples, dt0 = _problem()
    if grid == "scaled":
        dt0 = -1.0  # the scaled stable step per sample, last step shortened
    with _lib.Handle(an.n, "f32") as h:
        h.set_anatomy(an.p_w, an.p_g)
        h.set_observations(obs.pet, obs.t1, obs.t2, obs.points, LIK, step_pet=1, step_ti=1)
        ll, ga = h.adjoint_grad(samples, dt0, an.L, state=state)
        gf = _fd(h, samples, dt0, an.L, "f64")
    err, a, f = _rel_err(ga, gf, samples)
    for s in range(len(samples)):
        print(f"{state} {grid} sample {s}: rel err {err[s]:.2e}")
        for i in range(6):
            print(f"   {NAMES[i]:4s} adjoint {a[s, i]: .6e}  fd {f[s, i]: .6e}")
    assert np.all(np.isfinite(ll)) and np.all(err <= tol)


def test_adjoint_is_independent_of_checkpoint_interval(gbg):
    an, obs, samples, dt0 = _problem()
    with _lib.Handle(an.n, "f32") as h:
        h.set_anatomy(an.p_w, an.p_g)
        h.set_observations(obs.pet, obs.t1, obs.t2, obs.points, LIK, step_pet=1, step_ti=1)
        ref = h.adjoint_grad(samples, dt0, an.L, checkpoint_every=50)
        for k in (1, 7, 13):
            got = h.adjoint_grad(samples, dt0, an.L, checkpoint_every=k)
            assert np.array_equal(got[0], ref[0])
            assert np.allclose(got[1], ref[1], rtol=1e-12, atol=0)


def test_adjoint_argument_errors(gbg):
    an, obs, samples, dt0 = _problem()
    with _lib.Handle(an.n, "f32") as h:
        with pytest.raises(_lib.GbgError) as e:
            h.adjoint_grad(samples, dt0, an.L)  # no anatomy / observations
        assert e.value.status == -5
        h.set_anatomy(an.p_w, an.p_g)
        h.set_observations(obs.pet, obs.t1, obs.t2, obs.points, LIK)
        for bad_dt0 in (0.0, -2.0):  # no grid; scaled grid beyond the stability limit
            with pytest.raises(_lib.GbgError):
                h.adjoint_grad(samples, bad_dt0, an.L)
        bad = [(np.nan,) + samples[0][1:]]
        with pytest.raises(_lib.GbgError):
            h.adjoint_grad(bad, dt0, an.L)


def test_batched_smooth_grid_equals_adjoint_forward(gbg):
    """The batched population solver on the smooth time grid (dt0 > 0) and
    the adjoint's float forward pass are the same model: log L bit for bit;
    the last, shortened step is taken (log L differs between tend and a tend
    a fraction of a step later)."""
    an, obs, samples, dt0 = _problem()
    extra = [(0.0009, 0.03, 16.1, 15.2, 15.8, 3.0 * dt0), (0.0017, 0.09, 15.0, 16.0, 15.0, 0.4 * dt0)]
    smp = samples + extra
    with _lib.Handle(an.n, "f32", max_samples=8) as h:
        h.set_anatomy(an.p_w, an.p_g)
        h.set_observations(obs.pet, obs.t1, obs.t2, obs.points, LIK, step_pet=1, step_ti=1)
        ll_adj, _ = h.adjoint_grad(smp, dt0, an.L, state="f32", want_grad=False)
        r = h.batch_solve(smp, an.L, dt0=dt0)
        ll_pop = np.array([d["total"] for d in r["loglik"]])
        assert np.array_equal(ll_adj, ll_pop), (ll_adj, ll_pop)
        assert list(r["nsteps"]) == [int(np.ceil(s[5] / dt0)) for s in smp]
        later = [s[:5] + (s[5] + 0.3 * dt0,) for s in smp]
        ll_later = np.array([d["total"] for d in h.batch_solve(later, an.L, dt0=dt0)["loglik"]])
        assert np.all(ll_later != ll_pop)
        # the reference schedule is still the default
        r0 = h.batch_solve(smp, an.L)
        k_ref = [S.num_steps(S.reference_dt(an.n, s[0], an.L)[0], s[5]) for s in smp]
        assert list(r0["nsteps"]) == k_ref


def test_scaled_grid_keeps_the_scaling_symmetry(gbg):
    """(Dw, rho, tend) -> (c Dw, c rho, tend / c) leaves the continuous
    model's density at tend unchanged; on the scaled grid (dt0 < 0) the
    discrete model keeps it up to float rounding of the coefficients, on the
    fixed grid it does not. Also: the batched solver equals the adjoint's
    forward pass bit for bit on the scaled grid."""
    an, obs, samples, dt0 = _problem()
    with _lib.Handle(an.n, "f32", max_samples=8) as h:
        h.set_anatomy(an.p_w, an.p_g)
        h.set_observations(obs.pet, obs.t1, obs.t2, obs.points, LIK, step_pet=1, step_ti=1)
        base = samples[0]
        scaled = [base] + [(c * base[0], c * base[1], *base[2:5], base[5] / c) for c in (0.8, 1.25)]
        phi = h.batch_solve(scaled, an.L, with_loglik=False, want_phi=True, dt0=-1.0)["phi"]
        for k in (1, 2):
            rel = np.linalg.norm(phi[k] - phi[0]) / np.linalg.norm(phi[0])
            assert rel < 1e-5, rel
        phi_f = h.batch_solve(scaled, an.L, with_loglik=False, want_phi=True, dt0=dt0)["phi"]
        assert np.linalg.norm(phi_f[1] - phi_f[0]) / np.linalg.norm(phi_f[0]) > 1e-4
        ll_adj, _ = h.adjoint_grad(scaled, -1.0, an.L, state="f32", want_grad=False)
        ll_pop = np.array([d["total"] for d in h.batch_solve(scaled, an.L, dt0=-1.0)["loglik"]])
        assert np.array_equal(ll_adj, ll_pop)


def test_fused_backward_at_128_matches_fp64_adjoint(gbg):
    """At 128^3 the float path runs the fused backward kernel over the samples
    still running at each step (samples reordered by step count inside the
    library); the FP64-state path runs the separate kernels. Three samples of
    different lengths, given out of order: the float gradient agrees with the
    FP64 one to 1e-3 (relative sensitivities theta_i dlogL/dtheta_i), log L to
    1e-4 relative, and neither depends on the checkpoint interval."""
    n = 128
    an = S.make_anatomy(n, seed=4)
    c = (63.0, 64.5, 62.0)
    truth = np.clip(S.gaussian_ic(an, *c, peak=0.9, sigma=4.0), 0, 1)
    obs = S.make_observations(truth, an, seed=3, centre_xyz=c, radius_vox=20.0)
    samples = [(0.0013, 0.05, 63.3, 64.2, 62.6, 24.3), (0.0021, 0.12, 62.6, 64.4, 62.3, 41.7),
               (0.0017, 0.08, 63.1, 64.9, 61.8, 33.0)]
    with _lib.Handle(n, "f32", max_samples=4) as h:
        h.set_anatomy(an.p_w, an.p_g)
        h.set_observations(obs.pet, obs.t1, obs.t2, obs.points, LIK)
        l32, g32 = h.adjoint_grad(samples, -1.0, an.L, state="f32")
        l32b, g32b = h.adjoint_grad(samples, -1.0, an.L, state="f32", checkpoint_every=7)
        l64, g64 = h.adjoint_grad(samples, -1.0, an.L, state="f64")
    err, a, f = _rel_err(g32, g64, samples)
    print("fused vs fp64 relative gradient error", err)
    assert np.all(err < 1e-3), (a, f)
    assert np.all(np.abs(l32 - l64) <= 1e-4 * np.abs(l64))
    assert np.array_equal(l32, l32b)
    assert np.allclose(g32, g32b, rtol=1e-9, atol=1e-12 * np.abs(g32).max())
