"""GPU: the learned surrogate (bf16 tensor-core 3D U-Net).

* input features against a NumPy restatement of their definition;
* loss and parameter gradient of one batch against the NumPy oracle of the
  same network (oracle/surrogate_oracle.py), which rounds to bf16 where the
  GPU stores bf16; the GPU accumulates in fp32 and the oracle in fp64, so the
  gradient agrees to a relative L2 error of 3e-2 (typically ~1e-3);
* training on solver outputs reduces the loss on those samples, and the
  trained surrogate's predicted density is close to the solver's;
* the surrogate's log-likelihood is the handle's likelihood of the
  surrogate's predicted density.
"""
import numpy as np
import pytest

from gliomauq_gb300 import _lib, synthetic as S
from oracle import surrogate_oracle as SO

pytestmark = pytest.mark.gpu
LIK = (0.0025, 1.0, 0.7, 0.25, 0.09)
N = 32


def _setup(h, an):
    lo = (S.PRIOR_DW_CM2[0], S.PRIOR_RHO[0], S.PRIOR_T[0])
    hi = (S.PRIOR_DW_CM2[1], S.PRIOR_RHO[1], S.PRIOR_T[1])
    return lo, hi


def _down2(phi):
    B, n = phi.shape[0], phi.shape[1]
    m = n // 2
    return phi.reshape(B, m, 2, m, 2, m, 2).astype(np.float64).mean(axis=(2, 4, 6))


def _features_np(an, samples, lo, hi):
    """Restatement of the surrogate's input channels (factor 2)."""
    n, m = an.n, an.n // 2
    pw = an.p_w.reshape(m, 2, m, 2, m, 2).mean(axis=(1, 3, 5))
    pg = an.p_g.reshape(m, 2, m, 2, m, 2).mean(axis=(1, 3, 5))
    z, y, x = np.meshgrid(np.arange(m), np.arange(m), np.arange(m), indexing="ij")
    px, py, pz = (x + 0.5) * 2 - 0.5, (y + 0.5) * 2 - 0.5, (z + 0.5) * 2 - 0.5
    out = np.zeros((len(samples), m, m, m, 16))
    for b, (Dw, rho, x0, y0, z0, T) in enumerate(samples):
        d2 = (px - x0) ** 2 + (py - y0) ** 2 + (pz - z0) ** 2
        dvox = Dw / an.L ** 2 * n * n
        front = 2.0 * np.sqrt(dvox * rho) * T
        out[b, ..., 0] = pw
        out[b, ..., 1] = pg
        out[b, ..., 2] = np.exp(-d2 / (2 * 1.5 ** 2))
        out[b, ..., 3] = (Dw - lo[0]) / (hi[0] - lo[0])
        out[b, ..., 4] = (rho - lo[1]) / (hi[1] - lo[1])
        out[b, ..., 5] = (T - lo[2]) / (hi[2] - lo[2])
        out[b, ..., 6] = (np.sqrt(d2) - front) / 16.0
    return out


@pytest.mark.parametrize("engine", ["mma.sync", "tcgen05"])
def test_features_and_gradient_vs_oracle(gbg, engine):
    an = S.make_anatomy(N, seed=5)
    samples = [p.as_tuple() for p in S.draw_prior(an, 2, seed=11)]
    with _lib.Handle(N, "f32", max_samples=4) as h:
        h.set_anatomy(an.p_w, an.p_g)
        lo, hi = _setup(h, an)
        sg = _lib.Surrogate(h, an.L, lo, hi, batch_max=4, seed=3)
        sg.set_engine(engine)
        try:
            f = sg.features(samples)
            ref = SO.bf16(_features_np(an, samples, lo, hi))
            # one bf16 ulp (2^-8 relative) for values rounded on either side of a tie
            assert np.all(np.abs(f - ref) <= 2.0 ** -7 * np.abs(ref) + 1e-6)

            rng = np.random.default_rng(2)
            targ = rng.uniform(0, 1, (2, N // 2, N // 2, N // 2)).astype(np.float32)
            params = sg.get_params()
            assert params.size == SO.offsets()[1] == sg.nparams()
            # nonzero biases so that the bias path is exercised
            offs, _ = SO.offsets()
            for k, (wo, bo) in enumerate(offs):
                co = SO.LAYERS[k][1]
                params[bo:bo + co] = rng.normal(0, 0.05, co)
            sg.set_params(params)
            loss, g = sg.loss_grad(samples, targ)
            loss_o, g_o = SO.loss_and_grad(params, f.astype(np.float64), targ.astype(np.float64))
            assert abs(loss - loss_o) <= 1e-3 * loss_o
            rel = np.linalg.norm(g - g_o) / np.linalg.norm(g_o)
            assert rel < 3e-2, rel
            # layer by layer: every layer's gradient block agrees in direction
            for k, (wo, bo) in enumerate(offs):
                a, b = g[wo:bo], g_o[wo:bo]
                if np.linalg.norm(b) > 0:
                    cos = a @ b / (np.linalg.norm(a) * np.linalg.norm(b))
                    assert cos > 0.995, (k, cos)
            # loss without gradient: the same sum (fp64 atomics, any order)
            loss2, _ = sg.loss_grad(samples, targ, want_grad=False)
            assert abs(loss2 - loss) <= 1e-12 * loss
        finally:
            sg.close()


def test_train_predict_and_loglik(gbg):
    an = S.make_anatomy(N, seed=5)
    train = [p.as_tuple() for p in S.draw_prior(an, 24, seed=21)]
    test = [p.as_tuple() for p in S.draw_prior(an, 4, seed=22)]
    with _lib.Handle(N, "f32", max_samples=24) as h:
        h.set_anatomy(an.p_w, an.p_g)
        lo, hi = _setup(h, an)
        sol = h.batch_solve(train[:4], an.L, with_loglik=False, want_phi=True)["phi"]
        targ = _down2(sol).astype(np.float32)
        u = h.batch_solve([test[0]], an.L, with_loglik=False, want_phi=True)["phi"][0]
        obs = S.make_observations(u.astype(np.float64), an, seed=3, centre_xyz=(15, 16, 15),
                                  radius_vox=9.0)
        h.set_observations(obs.pet, obs.t1, obs.t2, obs.points, LIK)
        sg = _lib.Surrogate(h, an.L, lo, hi, batch_max=8, seed=7)
        try:
            before, _ = sg.loss_grad(train[:4], targ, want_grad=False)
            last = sg.train(train, epochs=100, batch=8, lr=2e-3, seed=1)
            after, _ = sg.loss_grad(train[:4], targ, want_grad=False)
            print(f"surrogate loss before {before:.4g} after {after:.4g} last epoch {last:.4g}")
            assert np.isfinite(last) and after < 0.1 * before
            out = sg.loglik(test, want_phi=True)
            phi = out["phi"]
            assert phi.shape == (4, N, N, N) and np.isfinite(phi).all()
            assert np.all(phi[:, ~an.brain] == 0) and phi.min() >= 0 and phi.max() <= 1
            # predicted density vs the solver's on held-out samples
            true = h.batch_solve(test, an.L, with_loglik=False, want_phi=True)["phi"]
            err = np.linalg.norm(phi - true) / np.linalg.norm(true)
            print(f"surrogate held-out relative L2 error {err:.3f}")
            assert err < 0.5
            # the surrogate's log L is the likelihood of its predicted density
            for b in range(4):
                h.set_phi(phi[b].astype(np.float64))
                ref = h.loglik()["total"]
                got = out["loglik"][b]["total"]
                assert np.isfinite(got) and abs(got - ref) <= 1e-9 * max(1.0, abs(ref))
        finally:
            sg.close()


def test_surrogate_argument_errors(gbg):
    an = S.make_anatomy(N, seed=5)
    lo = (S.PRIOR_DW_CM2[0], S.PRIOR_RHO[0], S.PRIOR_T[0])
    hi = (S.PRIOR_DW_CM2[1], S.PRIOR_RHO[1], S.PRIOR_T[1])
    with _lib.Handle(N, "f64") as h:
        h.set_anatomy(an.p_w, an.p_g)
        with pytest.raises(_lib.GbgError):
            _lib.Surrogate(h, an.L, lo, hi)
    with _lib.Handle(N, "f32", max_samples=2) as h:
        h.set_anatomy(an.p_w, an.p_g)
        sg = _lib.Surrogate(h, an.L, lo, hi, batch_max=2)
        try:
            smp = [p.as_tuple() for p in S.draw_prior(an, 3, seed=1)]
            with pytest.raises(_lib.GbgError):
                sg.features(smp)  # B > batch_max
            with pytest.raises(_lib.GbgError):
                sg.loglik(smp[:1])  # no observations set
            bad = [tuple(np.nan if i == 1 else v for i, v in enumerate(smp[0]))]
            with pytest.raises(_lib.GbgError):
                sg.train(bad, epochs=1, batch=1)
        finally:
            sg.close()


def test_tcgen05_and_mma_sync_engines_agree(gbg):
    """The two convolution engines compute the same GEMMs with different
    fp32 summation orders: loss within 1e-5 relative, parameter gradient
    within 1e-2 relative L2 (bf16 rounding of the stored activations can
    differ by one unit), at 64^3 (32^3 surrogate grid, 4 samples)."""
    n = 64
    an = S.make_anatomy(n, seed=2)
    samples = [p.as_tuple() for p in S.draw_prior(an, 4, seed=12)]
    lo = (S.PRIOR_DW_CM2[0], S.PRIOR_RHO[0], S.PRIOR_T[0])
    hi = (S.PRIOR_DW_CM2[1], S.PRIOR_RHO[1], S.PRIOR_T[1])
    rng = np.random.default_rng(4)
    targ = rng.uniform(0, 1, (4, n // 2, n // 2, n // 2)).astype(np.float32)
    with _lib.Handle(n, "f32", max_samples=4) as h:
        h.set_anatomy(an.p_w, an.p_g)
        sg = _lib.Surrogate(h, an.L, lo, hi, batch_max=4, seed=9)
        try:
            res = {}
            for eng in ("mma.sync", "tcgen05"):
                sg.set_engine(eng)
                res[eng] = sg.loss_grad(samples, targ)
        finally:
            sg.close()
    (l0, g0), (l1, g1) = res["mma.sync"], res["tcgen05"]
    print("loss", l0, l1, "grad rel", np.linalg.norm(g1 - g0) / np.linalg.norm(g0))
    assert abs(l1 - l0) <= 1e-5 * abs(l0)
    assert np.linalg.norm(g1 - g0) <= 1e-2 * np.linalg.norm(g0)
