"""GPU: the CUDA step through the C ABI against the reference (golden
fixtures) and the oracle. Exact modes must be bit-identical; the fast FP32
path must stay within the stated error of the FP64 reference."""
import hashlib

import numpy as np
import pytest

from gliomauq_gb300 import _lib, synthetic as S
from helpers import boundary_layer, golden_json, golden_npz, rel_l2

pytestmark = pytest.mark.gpu

# Fast FP32 path: relative L2 error of the final density against the FP64
# reference after a full config-1 solve (64^3, 237 steps).
F32_REL_L2_TOL = 1e-5


def _sha(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<f8").tobytes()).hexdigest()


@pytest.mark.parametrize("k", [1, 10, 60])
@pytest.mark.parametrize("prec,variant", [("f64", "f64"), ("f32ref", "f32")])
def test_exact_modes_bitwise_vs_reference_golden(gbg, prec, variant, k):
    d = golden_npz("rd32.npz")
    with _lib.Handle(32, prec) as h:
        h.set_anatomy(d["p_w"], d["p_g"])
        h.set_phi(d["phi0"])
        h.rd_step(float(d[f"Dw_{variant}"]), float(d[f"Dg_{variant}"]), float(d["rho"]),
                  float(d[f"dt_{variant}"]), k)
        out = h.get_phi()
    assert np.array_equal(out, d[f"phi_{variant}_{k}"].astype(np.float64))


@pytest.mark.parametrize("prec,variant", [("f64", "f64"), ("f32ref", "f32")])
def test_config1_full_run_bitwise(gbg, prec, variant):
    meta = golden_json("c1_64.json")
    a = golden_npz("anatomy64.npz")
    with _lib.Handle(64, prec) as h:
        h.set_anatomy(a["p_w"], a["p_g"])
        h.set_phi(a["phi0"])
        ns, dt = h.run(meta["Dw_file"], meta["rho"], meta["tend"], meta["L"])
        out = h.get_phi()
    assert ns == meta[variant]["steps"] and dt == meta[variant]["dt"]
    assert _sha(out) == meta[variant]["sha256"]


def test_fast_f32_error_against_fp64_reference(gbg, oracle_lib):
    meta = golden_json("c1_64.json")
    a = golden_npz("anatomy64.npz")
    with _lib.Handle(64, "f32") as h:
        h.set_anatomy(a["p_w"], a["p_g"])
        h.set_phi(a["phi0"])
        ns, dt = h.run(meta["Dw_file"], meta["rho"], meta["tend"], meta["L"])
        out = h.get_phi()
    assert ns == 237 and dt == meta["f64"]["dt"]
    dt64, dw, dg = S.reference_dt(64, meta["Dw_file"], meta["L"])
    ref = oracle_lib.rd_solve(a["p_w"], a["p_g"], a["phi0"], dw, dg, meta["rho"], dt64, ns)
    assert _sha(ref) == meta["f64"]["sha256"]
    err = rel_l2(out, ref)
    print(f"fast f32 vs FP64 reference, config 1: rel L2 = {err:.3e}")
    assert err <= F32_REL_L2_TOL
    brain = (a["p_w"].astype(np.float64) + a["p_g"]) > 0
    assert np.all(out[boundary_layer(brain)] == 0.0) and np.all(out[~brain] == 0.0)


@pytest.mark.parametrize("prec", ["f64", "f32ref"])
@pytest.mark.parametrize("seed", [0, 1])
def test_exact_modes_vs_live_oracle_random(gbg, oracle_lib, prec, seed):
    """Random anatomy (including non-tissue holes), random densities with values
    below 0 and above 1, odd grid size: bitwise equal to the oracle."""
    rng = np.random.default_rng(seed)
    n = 24 + 3 * seed
    pw = rng.random((n, n, n)) * (rng.random((n, n, n)) > 0.15)
    pg = (1 - pw) * (rng.random((n, n, n)) > 0.1)
    phi = rng.uniform(-0.2, 1.2, size=(n, n, n))
    if prec == "f32ref":
        pw, pg, phi = (x.astype(np.float32).astype(np.float64) for x in (pw, pg, phi))
    Dw, Dg, rho, dt = 2.1e-4, 2.1e-5, 0.08, 0.5 * (1 / n) ** 2 / (6 * 2.1e-4)
    with _lib.Handle(n, prec) as h:
        h.set_anatomy(pw, pg)
        h.set_phi(phi)
        h.rd_step(Dw, Dg, rho, dt, 7)
        out = h.get_phi()
    ref = oracle_lib.rd_solve(pw, pg, phi, Dw, Dg, rho, dt, 7, prec=prec)
    assert np.array_equal(out, ref.astype(np.float64))


@pytest.mark.parametrize("prec", ["f64", "f32ref", "f32"])
def test_zero_state_stays_zero_and_full_tissue(gbg, prec):
    n = 32
    with _lib.Handle(n, prec) as h:
        h.set_anatomy(np.full((n,) * 3, 0.6), np.full((n,) * 3, 0.4))
        h.set_phi(np.zeros((n,) * 3))
        h.rd_step(1e-4, 1e-5, 0.1, 1.0, 3)
        assert np.all(h.get_phi() == 0.0)
        # uniform density in an all-tissue periodic box follows the logistic ODE
        h.set_phi(np.full((n,) * 3, 0.25))
        h.rd_step(1e-4, 1e-5, 0.1, 1.0, 1)
        u = h.get_phi()
    exp = 0.25 + 1.0 * 0.1 * 0.25 * 0.75
    assert np.allclose(u, exp, rtol=1e-6)


def test_errors_are_reported(gbg):
    with _lib.Handle(32, "f64") as h:
        with pytest.raises(_lib.GbgError) as e:
            h.rd_step(1e-4, 1e-5, 0.1, 1.0, 1)  # before anatomy/phi
        assert e.value.status == -5
        with pytest.raises(_lib.GbgError) as e:
            h.set_anatomy(np.full((32,) * 3, np.nan), np.zeros((32,) * 3))
        assert e.value.status == -4
        with pytest.raises(ValueError):
            h.set_phi(np.zeros(10))
    with pytest.raises(_lib.GbgError) as e:
        _lib.Handle(2, "f64")
    assert e.value.status == -1
