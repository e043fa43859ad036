"""GPU: the multiresolution-grid kernels through the C ABI, on MRAG ghost
tables of a mixed-level grid, against the reference (golden) and the AMR
oracle (random fields on the same grid): bitwise in both exact modes."""
import numpy as np
import pytest

from gliomauq_gb300 import _lib
from helpers import golden_npz
from oracle import amr_oracle as A

pytestmark = pytest.mark.gpu
PREC = {"f64": "f64", "f32": "f32ref"}
REAL = {"f64": np.float64, "f32": np.float32}


def load(h, d, phi=None):
    h.set_grid(d["blocks"], d["p_w"], d["p_g"], d["phi"] if phi is None else phi)
    h.set_ghosts(d["ghost_start"], d["ghost_src_block"], d["ghost_src_cell"].astype(np.int32),
                 d["ghost_w"].astype(np.float64))


@pytest.mark.parametrize("variant", ["f64", "f32"])
def test_amr_step_matches_reference(gbg, variant):
    d = golden_npz(f"amr64_{variant}.npz")
    with _lib.AmrHandle(64, PREC[variant]) as h:
        load(h, d)
        h.step(float(d["Dw"]), float(d["Dg"]), float(d["rho"]), float(d["dt"]),
               int(d["steps_after"]))
        out = h.get_phi()
    assert np.array_equal(out, d["phi_after"])


@pytest.mark.parametrize("variant", ["f64", "f32"])
def test_amr_fwt_matches_reference(gbg, variant):
    d = golden_npz(f"amr64_{variant}.npz")
    with _lib.AmrHandle(64, PREC[variant]) as h:
        load(h, d)
        got = h.fwt_detail()
    assert np.array_equal(got, d["fwt"])


@pytest.mark.parametrize("variant", ["f64", "f32"])
def test_amr_random_fields_match_oracle(gbg, variant):
    d = golden_npz(f"amr64_{variant}.npz")
    real = REAL[variant]
    rng = np.random.default_rng(9)
    phi = rng.uniform(-0.1, 1.1, size=d["phi"].shape).astype(real).astype(np.float64)
    tabs = (d["ghost_start"], d["ghost_src_block"], d["ghost_src_cell"].astype(np.int32),
            d["ghost_w"].astype(np.float64))
    with _lib.AmrHandle(64, PREC[variant]) as h:
        load(h, d, phi)
        det = h.fwt_detail()
        h.step(2e-4, 2e-5, 0.2, 0.5, 3)
        out = h.get_phi()
    assert np.array_equal(det, A.fwt_detail(phi.reshape(-1, 4096), tabs, real))
    ref = phi.reshape(-1, 4096)
    for _ in range(3):
        ref = A.step(d["blocks"][:, 0], d["p_w"].reshape(-1, 4096), d["p_g"].reshape(-1, 4096), ref,
                     tabs, 2e-4, 2e-5, 0.2, 0.5, real).reshape(-1, 4096)
    assert np.array_equal(out.reshape(-1, 4096), ref.astype(np.float64))


def test_amr_argument_errors(gbg):
    d = golden_npz("amr64_f64.npz")
    with _lib.AmrHandle(8, "f64") as h:
        with pytest.raises(_lib.GbgError):
            h.set_grid(d["blocks"], d["p_w"], d["p_g"], d["phi"])  # more blocks than capacity
        with pytest.raises(_lib.GbgError):
            h.step(1e-4, 1e-5, 0.1, 1.0, 1)  # no ghost tables
    with _lib.AmrHandle(64, "f64") as h:
        h.set_grid(d["blocks"], d["p_w"], d["p_g"], d["phi"])
        bad = d["ghost_src_block"].copy()
        bad[0] = 10_000
        with pytest.raises(_lib.GbgError):
            h.set_ghosts(d["ghost_start"], bad, d["ghost_src_cell"].astype(np.int32),
                         d["ghost_w"].astype(np.float64))


@pytest.mark.parametrize("variant", ["f64", "f32"])
def test_amr_remap_matches_reference_regrid(gbg, variant):
    """The forced regrid of the reference (3 blocks split by BlockSplitter, one
    group collapsed by BlockCollapser) as one gbg_amr_remap on the GPU."""
    d = golden_npz(f"amr64_{variant}.npz")
    kind, src = A.remap_plan(d["blocks"], d["s2_blocks"])
    with _lib.AmrHandle(96, PREC[variant]) as h:
        load(h, d, d["phi_after"])
        h.remap(d["s2_blocks"], kind, src)
        out = h.get_phi()
        with pytest.raises(_lib.GbgError):
            h.step(1e-4, 1e-5, 0.1, 1.0, 1)  # the new grid needs its ghost tables
    assert np.array_equal(out, d["s2_phi"])


def test_amr_dump_matches_oracle(gbg):
    d = golden_npz("amr64_f64.npz")
    with _lib.AmrHandle(64, "f64") as h:
        load(h, d)
        u = h.dump_uniform(64)
        u2 = h.dump_uniform(32, reference_rules=False)
    assert np.array_equal(u, A.dump_uniform(d["blocks"], d["phi"], 64))
    assert np.array_equal(u2, A.dump_uniform(d["blocks"], d["phi"], 32, reference_rules=False))
