"""GPU: the adaptive solve through the library (gbg_amr_run: the
Glioma_HG_UQ::run loop with automatic regrids on the device grid, ghost
tables compiled by the library) against the reference's own adaptive runs,
bit for bit in both exact modes; and the fast FP32 mode's error against FP64
on the same adaptive configuration."""
import os
import sys

import numpy as np
import pytest

from gliomauq_gb300 import _lib, amr, synthetic as S
from helpers import golden_json, golden_npz

pytestmark = pytest.mark.gpu
PREC = {"f64": "f64", "f32": "f32ref"}

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
from make_golden import ADAPTIVE64, adaptive_phi_sha  # noqa: E402


def _input64(seed_xyz=(20.3, 24.6, 22.1), peak=0.5, sigma=1.5):
    a = golden_npz("anatomy64.npz")
    pw, pg = a["p_w"].astype(np.float64), a["p_g"].astype(np.float64)
    an = S.Anatomy(n=64, p_w=pw, p_g=pg, psi=None)
    phi0 = S.gaussian_ic(an, *seed_xyz, peak=peak, sigma=sigma).astype(np.float32)
    return (amr.to_block_major(pw, 2), amr.to_block_major(pg, 2),
            amr.to_block_major(phi0.astype(np.float64), 2))


@pytest.mark.parametrize("variant", ["f64", "f32"])
def test_library_ghost_tables_step_like_the_reference_tables(gbg, variant):
    """The mixed-level grid of amr64_*.npz stepped 10 times with the tables
    the library compiles (gbg_amr_build_ghosts) equals the reference."""
    d = golden_npz(f"amr64_{variant}.npz")
    with _lib.AmrHandle(len(d["blocks"]), PREC[variant]) as h:
        h.set_grid(d["blocks"], d["p_w"], d["p_g"], d["phi"])
        h.build_ghosts()
        h.step(float(d["Dw"]), float(d["Dg"]), float(d["rho"]), float(d["dt"]),
               int(d["steps_after"]))
        out = h.get_phi()
    assert np.array_equal(out, d["phi_after"])


@pytest.mark.parametrize("variant", ["f64", "f32"])
def test_adaptive_run_matches_reference_state(gbg, variant):
    """gbg_amr_run on the input of amr64_*.npz (regrid every 25 days to 60,
    no final refinement): the reference's blocks and densities bit for bit."""
    d = golden_npz(f"amr64_{variant}.npz")
    pw, pg, phi = _input64()
    with _lib.AmrHandle(512, PREC[variant]) as h:
        h.set_grid(amr.uniform_blocks(2), pw, pg, phi)
        steps, regrids = h.run(0.0013, 0.1, 60.0, 6.4, bpd=4, dumpfreq=25.0, adaptive=True,
                               max_level=2, final_refine=False)
        blocks = h.blocks()
        out = h.get_phi()
    assert regrids == 2
    ref = {tuple(b): i for i, b in enumerate(d["blocks"].tolist())}
    assert set(map(tuple, blocks.tolist())) == set(ref)
    for i, b in enumerate(blocks.tolist()):
        assert np.array_equal(out[i], d["phi"][ref[tuple(b)]]), b


@pytest.mark.parametrize("variant", ["f64", "f32"])
def test_long_adaptive_run_matches_reference(gbg, variant):
    """tests/golden/adaptive64.json: regrids every 10 days to 110 days with
    refinements and compressions, then the final refinement: same counts,
    blocks and densities (hash) as the reference's run."""
    c = ADAPTIVE64
    ref = golden_json("adaptive64.json")[variant]
    pw, pg, phi = _input64(tuple(c["seed_xyz"]), c["peak"], c["sigma"])
    with _lib.AmrHandle(512, PREC[variant]) as h:
        h.set_grid(amr.uniform_blocks(2), pw, pg, phi)
        steps, regrids = h.run(c["Dw"], c["rho"], c["tend"], c["L"], bpd=c["bpd"],
                               dumpfreq=c["dumpfreq"], adaptive=True, max_level=c["max_level"])
        blocks = h.blocks()
        out = h.get_phi()
    assert (steps, regrids) == (ref["steps"], ref["regrids"])
    assert sorted(blocks.tolist()) == ref["blocks"]
    assert adaptive_phi_sha(blocks.tolist(), out) == ref["phi_sha256"]


def test_adaptive_run_without_regrids_equals_uniform_solver(gbg):
    """adaptive = 0 (the reference's -adaptive 0): the one-level block grid
    takes the reference's steps and equals the uniform exact solver."""
    pw, pg, phi = _input64()
    with _lib.AmrHandle(64, "f64") as h:
        h.set_grid(amr.uniform_blocks(2), pw, pg, phi)
        steps, regrids = h.run(0.0013, 0.1, 30.0, 6.4, bpd=4)
        out = amr.from_block_major(h.get_phi(), 2)
    assert regrids == 0
    with _lib.Handle(64, "f64") as u:
        u.set_anatomy(amr.from_block_major(pw, 2), amr.from_block_major(pg, 2))
        u.set_phi(amr.from_block_major(phi, 2))
        k, _ = u.run(0.0013, 0.1, 30.0, 6.4)
        ref = u.get_phi()
    assert steps == k
    assert np.array_equal(out, ref)


def test_fast_f32_adaptive_error_against_f64(gbg):
    """The fast FP32 mode through the same adaptive loop: its uniform dump
    within 1e-4 relative L2 of the FP64 exact run's (its regrid decisions
    compare FP32 details with the tolerances, so the grids may differ)."""
    c = ADAPTIVE64
    pw, pg, phi = _input64(tuple(c["seed_xyz"]), c["peak"], c["sigma"])
    dumps = {}
    for prec in ("f64", "f32"):
        with _lib.AmrHandle(512, prec) as h:
            h.set_grid(amr.uniform_blocks(2), pw, pg, phi)
            h.run(c["Dw"], c["rho"], c["tend"], c["L"], bpd=c["bpd"], dumpfreq=c["dumpfreq"],
                  adaptive=True, max_level=c["max_level"])
            dumps[prec] = h.dump_uniform(64, reference_rules=False)
    err = np.linalg.norm(dumps["f32"] - dumps["f64"]) / np.linalg.norm(dumps["f64"])
    print(f"fast FP32 adaptive run vs FP64: rel L2 {err:.3e}")
    assert err <= 1e-4


def test_adaptive_run_argument_errors(gbg):
    pw, pg, phi = _input64()
    with _lib.AmrHandle(8, "f64") as h:
        with pytest.raises(_lib.GbgError):
            h.run(0.0013, 0.1, 30.0, 6.4, bpd=4)  # no grid set
        with pytest.raises(_lib.GbgError):
            h.set_grid(amr.uniform_blocks(2), pw, pg, phi)  # 64 blocks > max_blocks 8
