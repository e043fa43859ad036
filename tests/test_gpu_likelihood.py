"""GPU: the log-likelihood kernels through the C ABI against the reference's
`likelihood` program (golden, printed to six decimals) and the oracle."""
import numpy as np
import pytest

from gliomauq_gb300 import _lib
from helpers import golden_json, golden_npz

pytestmark = pytest.mark.gpu

# double accumulation in a fixed tree order against the reference's long
# double running sum
REL_TOL = 1e-11


@pytest.mark.parametrize("mode", ["sel", "all"])
def test_loglik_vs_reference_program(gbg, mode):
    d = golden_npz("lik32.npz")
    ref = golden_json("lik32.json")
    with _lib.Handle(32, "f64") as h:
        h.set_phi(d["model"])
        h.set_observations(d["pet"], d["t1"], d["t2"], d["points"], ref["params"],
                           step_pet=ref["step_pet"], step_ti=ref["step_ti"],
                           selective=(mode == "sel"))
        r = h.loglik()
    exp = ref[mode]
    assert r["n_pet"] == exp["n_pet"]
    for k in ("l_pet", "l_t1", "l_t2"):
        assert abs(r[k] - exp[k]) <= 1e-6, k
    assert abs(-r["total"] - exp["minus_loglik"]) <= 1e-6


@pytest.mark.parametrize("prec", ["f64", "f32ref", "f32"])
@pytest.mark.parametrize("selective", [True, False])
def test_loglik_vs_oracle(gbg, oracle_lib, prec, selective):
    d = golden_npz("lik32.npz")
    ref = golden_json("lik32.json")
    model = d["model"]
    if prec != "f64":
        model = model.astype(np.float32).astype(np.float64)
    with _lib.Handle(32, prec) as h:
        h.set_phi(model)
        h.set_observations(d["pet"], d["t1"], d["t2"], d["points"], ref["params"], step_pet=3,
                           step_ti=2, selective=selective)
        r = h.loglik()
    o = oracle_lib.loglik(model, d["pet"], d["t1"], d["t2"], d["points"], ref["params"],
                          step_pet=3, step_ti=2, selective=selective)
    assert r["n_pet"] == o["n_pet"]
    for k in ("l_pet", "l_t1", "l_t2", "total"):
        assert abs(r[k] - o[k]) <= REL_TOL * max(1.0, abs(o[k])), (k, r[k], o[k])


def test_loglik_edge_cases(gbg, oracle_lib):
    n = 32
    rng = np.random.default_rng(5)
    model = rng.random((n, n, n))
    pet = np.zeros((n, n, n))  # no PET voxel: N = 0, PET term 0
    t1 = (rng.random((n, n, n)) > 0.5).astype(float)
    t2 = np.ones((n, n, n))
    model[0, 0, 0] = 0.7  # u == uc: sgn = 0, alpha = 0.5
    params = (0.0025, 1.0, 0.7, 0.25, 0.09)
    pts = np.array([[0, 0, 0], [2, 4, 6], [31, 31, 31]], dtype=float)
    with _lib.Handle(n, "f64") as h:
        h.set_phi(model)
        h.set_observations(pet, t1, t2, pts, params, step_pet=3, step_ti=1, selective=True)
        r = h.loglik()
        with pytest.raises(_lib.GbgError):
            h.set_observations(pet, t1, t2, np.array([[40.0, 0, 0]]), params)
    o = oracle_lib.loglik(model, pet, t1, t2, pts, params, step_pet=3, step_ti=1, selective=True)
    assert r["n_pet"] == 0 and r["l_pet"] == 0.0
    for k in ("l_t1", "l_t2", "total"):
        assert abs(r[k] - o[k]) <= REL_TOL * max(1.0, abs(o[k]))
