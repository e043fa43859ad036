"""GPU: the MALA variant (gbg_mala_step, gbg_run_mala): phi and the slopes
sRho, sD of Glioma_MALA_SlopesOperator.h through the C ABI, bit-identical to
the reference (golden fixtures from the reference compiled in place) and to
the oracle restatement on random inputs."""
import numpy as np
import pytest

from gliomauq_gb300 import _lib
from helpers import golden_npz

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("k", [1, 40])
@pytest.mark.parametrize("prec,variant", [("f64", "f64"), ("f32ref", "f32")])
def test_mala_bitwise_vs_reference_golden(gbg, prec, variant, k):
    d = golden_npz("mala32.npz")
    with _lib.Handle(32, prec) as h:
        h.set_anatomy(d["p_w"], d["p_g"])
        h.set_phi(d["phi0"])
        h.mala_step(float(d[f"Dw_{variant}"]), float(d[f"Dg_{variant}"]), float(d["rho"]),
                    float(d[f"dt_{variant}"]), k)
        phi = h.get_phi()
        sr, sd = h.get_slopes()
    assert np.array_equal(phi, d[f"phi_{variant}_{k}"].astype(np.float64))
    assert np.array_equal(sr, d[f"sRho_{variant}_{k}"].astype(np.float64))
    assert np.array_equal(sd, d[f"sD_{variant}_{k}"].astype(np.float64))


@pytest.mark.parametrize("prec", ["f64", "f32ref"])
def test_mala_vs_live_oracle_random(gbg, oracle_lib, prec):
    """Random anatomy with holes, densities outside [0, 1], nonzero starting
    slopes, odd grid size: bitwise equal to the oracle."""
    rng = np.random.default_rng(7)
    n = 27
    pw = rng.random((n, n, n)) * (rng.random((n, n, n)) > 0.15)
    pg = (1 - pw) * (rng.random((n, n, n)) > 0.1)
    phi = rng.uniform(-0.2, 1.2, size=(n, n, n))
    sr0 = rng.normal(0, 3, size=(n, n, n))
    sd0 = rng.normal(0, 50, size=(n, n, n))
    if prec == "f32ref":
        pw, pg, phi, sr0, sd0 = (x.astype(np.float32).astype(np.float64)
                                 for x in (pw, pg, phi, sr0, sd0))
    Dw, Dg, rho, dt = 2.1e-4, 2.1e-5, 0.08, 0.5 * (1 / n) ** 2 / (6 * 2.1e-4)
    with _lib.Handle(n, prec) as h:
        h.set_anatomy(pw, pg)
        h.set_phi(phi)
        h.set_slopes(sr0, sd0)
        h.mala_step(Dw, Dg, rho, dt, 5)
        out = h.get_phi()
        sr, sd = h.get_slopes()
    ref = oracle_lib.mala_solve(pw, pg, phi, Dw, Dg, rho, dt, 5, prec=prec, sr0=sr0, sd0=sd0)
    for a, b in zip((out, sr, sd), ref):
        assert np.array_equal(a, b.astype(np.float64))


def test_run_mala_matches_steps_and_plain_run(gbg):
    """gbg_run_mala takes gbg_run's step count and dt, and its phi equals the
    plain run's (the slopes do not feed back into phi)."""
    d = golden_npz("mala32.npz")
    with _lib.Handle(32, "f64") as h:
        h.set_anatomy(d["p_w"], d["p_g"])
        h.set_phi(d["phi0"])
        ns, dt = h.run_mala(float(d["Dw_file"]), float(d["rho"]), 20.0, float(d["L"]))
        phi_m = h.get_phi()
        sr, sd = h.get_slopes()
        h.set_phi(d["phi0"])
        ns2, dt2 = h.run(float(d["Dw_file"]), float(d["rho"]), 20.0, float(d["L"]))
        phi_p = h.get_phi()
    assert (ns, dt) == (ns2, dt2) and ns > 0
    assert np.array_equal(phi_m, phi_p)
    assert np.isfinite(sr).all() and np.isfinite(sd).all() and np.abs(sr).max() > 0


def test_mala_errors(gbg):
    with _lib.Handle(16, "f32") as h:
        h.set_anatomy(np.ones((16,) * 3), np.zeros((16,) * 3))
        h.set_phi(np.zeros((16,) * 3))
        with pytest.raises(_lib.GbgError):
            h.mala_step(1e-4, 1e-5, 0.1, 0.1, 1)
    with _lib.Handle(16, "f64") as h:
        with pytest.raises(_lib.GbgError):
            h.get_slopes()  # not set
        h.set_anatomy(np.ones((16,) * 3), np.zeros((16,) * 3))
        with pytest.raises(_lib.GbgError):
            h.mala_step(1e-4, 1e-5, 0.1, 0.1, 1)  # phi not set
        h.set_phi(np.zeros((16,) * 3))
        with pytest.raises(_lib.GbgError):
            h.set_slopes(np.full((16,) * 3, np.nan), None)
        with pytest.raises(_lib.GbgError):
            h.mala_step(-1.0, 1e-5, 0.1, 0.1, 1)
