"""CPU: the AMR oracle restatement against the reference's adaptive-grid
outputs (tests/golden/amr64_*.npz, made from oracle/_ref): ghost layout,
10 steps on a mixed-level grid, and the FWT detail maxima -- bitwise."""
import numpy as np
import pytest

from helpers import golden_json, golden_npz
from oracle import amr_oracle as A

REAL = {"f64": np.float64, "f32": np.float32}


def tables(d):
    return (d["ghost_start"], d["ghost_src_block"], d["ghost_src_cell"].astype(np.int32),
            d["ghost_w"].astype(np.float64))


def test_fixture_grid_is_mixed_level_with_interpolated_ghosts():
    d = golden_npz("amr64_f64.npz")
    assert set(d["blocks"][:, 0].tolist()) == {1, 2}
    counts = np.diff(d["ghost_start"])
    assert counts.size == d["blocks"].shape[0] * A.NG
    assert {1, 2, 4, 8} <= set(counts.tolist())


@pytest.mark.parametrize("variant", ["f64", "f32"])
def test_amr_step_oracle_matches_reference(variant):
    d = golden_npz(f"amr64_{variant}.npz")
    real = REAL[variant]
    phi = d["phi"].reshape(-1, 4096)
    for _ in range(int(d["steps_after"])):
        phi = A.step(d["blocks"][:, 0], d["p_w"].reshape(-1, 4096), d["p_g"].reshape(-1, 4096),
                     phi, tables(d), float(d["Dw"]), float(d["Dg"]), float(d["rho"]),
                     float(d["dt"]), real).reshape(-1, 4096)
    assert np.array_equal(phi.reshape(d["phi_after"].shape).astype(np.float64), d["phi_after"])


@pytest.mark.parametrize("variant", ["f64", "f32"])
def test_amr_fwt_oracle_matches_reference(variant):
    d = golden_npz(f"amr64_{variant}.npz")
    got = A.fwt_detail(d["phi"].reshape(-1, 4096), tables(d), REAL[variant])
    assert np.array_equal(got, d["fwt"])


@pytest.mark.parametrize("variant", ["f64", "f32"])
def test_amr_remap_oracle_matches_reference(variant):
    """BlockSplitter + BlockCollapser of the forced regrid S1 -> S2."""
    d = golden_npz(f"amr64_{variant}.npz")
    real = REAL[variant]
    kind, src = A.remap_plan(d["blocks"], d["s2_blocks"])
    assert {0, 1, 2} <= set(kind.tolist())
    for name, key in (("phi_after", "s2_phi"), ("p_w", "s2_p_w"), ("p_g", "s2_p_g")):
        f = d[name].reshape(-1, 4096)
        g = A.ghost_values(f, *tables(d)[:3], tables(d)[3], real)
        out = A.remap(f, g, kind, src, real)
        assert np.array_equal(out.astype(np.float64), d[key]), name


def _sha(a):
    import hashlib
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<f8").tobytes()).hexdigest()


def test_amr_dump_oracle_matches_reference_dump():
    """oracle.amr_oracle.dump_uniform against the reference's own
    Glioma_HG_UQ::_dumpUQoutput (tests/golden/dump_ref.json, made by
    oracle/_ref/ref_dump_*): the adaptive 64^3 grid of amr64_f64.npz (levels
    1, 2), a 256^3 grid of levels 2, 3, 4, and a 256^3 grid of levels 1, 2
    whose level-1 cells the reference replicates 4^3 times where they cover
    8^3 (it leaves the rest of its output uninitialised; the hash covers the
    cells it writes)."""
    from oracle import refio
    ref = golden_json("dump_ref.json")
    d = golden_npz("amr64_f64.npz")
    u = A.dump_uniform(d["blocks"], d["phi"], 64)
    assert _sha(u) == ref["dump64"]["sha256"]
    assert np.count_nonzero(u) == ref["dump64"]["nonzero"]
    for name in ("grid3", "grid12"):
        g = ref[name]
        bl = np.array(g["blocks"], dtype=np.int32)
        assert sorted(set(bl[:, 0].tolist())) == g["levels"]
        ph = refio.dumpgrid_phi(bl)
        u = A.dump_uniform(bl, ph, g["gpd"])
        written = A.dump_uniform(bl, np.ones_like(ph), g["gpd"]) != 0
        assert int(written.sum()) == g["written"]
        assert _sha(u[written]) == g["sha256_written"], name
    assert ref["grid12"]["written"] < 256 ** 3 == ref["grid3"]["written"]


def test_same_level_ghost_tables_are_periodic_copies():
    """gliomauq_gb300.amr.same_level_ghosts in the oracle's ghost order: every
    ghost of a one-level grid equals the periodic neighbour cell of the
    uniform field."""
    from gliomauq_gb300 import amr
    assert np.array_equal(amr.ghost_lab_coords()[:, ::-1] + 1,
                          np.argwhere(A.LAB_SLOTS >= 0)[np.argsort(A.LAB_SLOTS[A.LAB_SLOTS >= 0])])
    level = 1
    n = 16 << level
    rng = np.random.default_rng(0)
    u = rng.random((n, n, n))
    blocks = amr.uniform_blocks(level)
    f = amr.to_block_major(u, level)
    assert np.array_equal(amr.from_block_major(f, level), u)
    st, sb, sc, w = amr.same_level_ghosts(blocks)
    gv = A.ghost_values(f.reshape(-1, 4096), st, sb, sc, w, np.float64).reshape(-1, 1736)
    lab = amr.ghost_lab_coords()
    for bi, (lv, ix, iy, iz) in enumerate(blocks):
        gx = (ix * 16 + lab[:, 0]) % n
        gy = (iy * 16 + lab[:, 1]) % n
        gz = (iz * 16 + lab[:, 2]) % n
        assert np.array_equal(gv[bi], u[gz, gy, gx])
