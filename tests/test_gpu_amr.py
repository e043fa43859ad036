"""GPU: the multiresolution-grid kernels through the C ABI, on MRAG ghost
tables of a mixed-level grid, against the reference (golden) and the AMR
oracle (random fields on the same grid): bitwise in both exact modes."""
import numpy as np
import pytest

from gliomauq_gb300 import _lib
from helpers import golden_json, golden_npz
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


def _sha(a):
    import hashlib
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<f8").tobytes()).hexdigest()


@pytest.mark.parametrize("name", ["dump64", "grid3", "grid12"])
def test_amr_dump_matches_reference_dump(gbg, name):
    """gbg_amr_dump_uniform(reference_rules = 1) against the reference's own
    Glioma_HG_UQ::_dumpUQoutput (hashes in tests/golden/dump_ref.json): the
    adaptive 64^3 grid (levels 1, 2), a 256^3 grid of levels 2, 3, 4 and a
    256^3 grid of levels 1, 2, where the reference replicates a level-1 cell
    4^3 times over the 8^3 it covers. The reference leaves the cells it does
    not write uninitialised; the library writes 0 there."""
    from oracle import refio
    ref = golden_json("dump_ref.json")[name]
    if name == "dump64":
        d = golden_npz("amr64_f64.npz")
        bl, ph = d["blocks"], d["phi"]
    else:
        bl = np.array(ref["blocks"], dtype=np.int32)
        ph = refio.dumpgrid_phi(bl)
    zeros = np.zeros(ph.size)
    with _lib.AmrHandle(len(bl), "f64") as h:
        h.set_grid(bl, zeros, zeros, ph)
        u = h.dump_uniform(ref["gpd"])
    if "sha256" in ref:
        assert _sha(u) == ref["sha256"]
    if name != "dump64":
        written = A.dump_uniform(bl, np.ones_like(ph), ref["gpd"]) != 0
        assert int(written.sum()) == ref["written"]
        assert _sha(u[written]) == ref["sha256_written"]
        assert not u[~written].any()


@pytest.mark.parametrize("variant", ["f64", "f32"])
def test_one_level_block_grid_equals_uniform_solver(gbg, variant):
    """A grid of 4^3 blocks at level 2 with periodic same-level ghost tables
    (gliomauq_gb300.amr) steps to the same bits as the uniform 64^3 exact
    solver: both restate the reference's operator, and a one-level MRAG grid
    is a periodic uniform grid."""
    from gliomauq_gb300 import amr, synthetic as S
    level, n = 2, 64
    an = S.make_anatomy(n, seed=3)
    phi = np.clip(S.gaussian_ic(an, 30.2, 33.1, 31.5, peak=0.8, sigma=3.0), 0, 1)
    Dw, rho, dt, steps = 0.0013 / (n * 0.1) ** 2, 0.03, 0.7, 12
    Dg = 0.1 * Dw
    if variant == "f32":
        Dw, Dg = float(np.float32(Dw)), float(np.float32(np.float32(0.1) * np.float32(Dw)))
        phi = phi.astype(np.float32).astype(np.float64)
    with _lib.Handle(n, PREC[variant]) as h:
        h.set_anatomy(an.p_w, an.p_g)
        h.set_phi(phi)
        h.rd_step(Dw, Dg, rho, dt, steps)
        ref = h.get_phi()
    blocks = amr.uniform_blocks(level)
    with _lib.AmrHandle(len(blocks), PREC[variant]) as h:
        h.set_grid(blocks, amr.to_block_major(an.p_w, level), amr.to_block_major(an.p_g, level),
                   amr.to_block_major(phi, level))
        h.set_ghosts(*amr.same_level_ghosts(blocks))
        h.step(Dw, Dg, rho, dt, steps)
        out = amr.from_block_major(h.get_phi(), level)
    assert np.array_equal(out, ref)


def test_fast_f32_one_level_grid_equals_uniform_fast_path(gbg):
    """The fast FP32 block-grid mode (GBG_PREC_F32) on a one-level grid is
    the uniform fast path bit for bit (same coefficients, same operation
    order); the anatomy is given in float-representable values so that both
    paths start from the same numbers."""
    from gliomauq_gb300 import amr, synthetic as S
    level, n = 2, 64
    an = S.make_anatomy(n, seed=3)
    pw = an.p_w.astype(np.float32).astype(np.float64)
    pg = an.p_g.astype(np.float32).astype(np.float64)
    phi = np.clip(S.gaussian_ic(an, 30.2, 33.1, 31.5, peak=0.8, sigma=3.0), 0, 1)
    phi = phi.astype(np.float32).astype(np.float64)
    Dw, rho, dt, steps = 0.0013 / (n * 0.1) ** 2, 0.03, 0.7, 12
    with _lib.Handle(n, "f32") as h:
        h.set_anatomy(pw, pg)
        h.set_phi(phi)
        h.rd_step(Dw, 0.1 * Dw, rho, dt, steps)
        ref = h.get_phi()
    blocks = amr.uniform_blocks(level)
    with _lib.AmrHandle(len(blocks), "f32") as h:
        h.set_grid(blocks, amr.to_block_major(pw, level), amr.to_block_major(pg, level),
                   amr.to_block_major(phi, level))
        h.set_ghosts(*amr.same_level_ghosts(blocks))
        h.step(Dw, 0.1 * Dw, rho, dt, steps)
        out = amr.from_block_major(h.get_phi(), level)
    assert np.array_equal(out, ref)


def test_fast_f32_mixed_level_grid_error_against_f64(gbg):
    """Fast FP32 mode on the reference's mixed-level grid (resolution-jump
    ghosts from MRAG's tables): relative L2 error against the FP64 mode after
    the fixture's steps below 1e-5 (float arithmetic, as the uniform fast
    path's 3.5e-7)."""
    d = golden_npz("amr64_f64.npz")
    outs = {}
    for prec in ("f64", "f32"):
        with _lib.AmrHandle(64, prec) as h:
            load(h, d)
            h.step(float(d["Dw"]), float(d["Dg"]), float(d["rho"]), float(d["dt"]), int(d["steps_after"]))
            outs[prec] = h.get_phi()
    err = np.linalg.norm(outs["f32"] - outs["f64"]) / np.linalg.norm(outs["f64"])
    print("fast f32 vs f64 relative L2", err)
    assert 0 < err < 1e-5


@pytest.mark.parametrize("source", ["reference_tables", "library_tables"])
def test_fast_f32_fused_step_equals_separate_ghost_pass(gbg, source):
    """The fast FP32 step's two forms (gbg_amr_fast_variant: ghosts evaluated
    while the lab is filled with per-face tables, or a separate ghost pass
    with per-cell tables) give the same densities bit for bit on the
    reference's mixed-level grid, with MRAG's tables or the library's."""
    d = golden_npz("amr64_f64.npz")
    outs = []
    for variant in (0, 1):
        with _lib.AmrHandle(len(d["blocks"]), "f32") as h:
            h.set_fast_variant(variant)
            h.set_grid(d["blocks"], d["p_w"], d["p_g"], d["phi"])
            if source == "reference_tables":
                h.set_ghosts(d["ghost_start"], d["ghost_src_block"], d["ghost_src_cell"], d["ghost_w"])
            else:
                h.build_ghosts()
            h.step(float(d["Dw"]), float(d["Dg"]), float(d["rho"]), float(d["dt"]), 25)
            outs.append(h.get_phi())
    assert np.array_equal(outs[0], outs[1])
    assert np.abs(outs[0]).max() > 0
