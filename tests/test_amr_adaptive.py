"""CPU: the adaptive grid's host logic in the library (gbg_amr_ghost_tables,
gbg_amr_plan_refine, gbg_amr_plan_compress; no GPU needed) against the
reference compiled in place:

  * the ghost instruction tables the library compiles equal MRAG's own
    (MRAG_BBInfoCreator through Grid::getBoundaryInfo) entry for entry -- same
    sources, same order, same weights -- on the adaptive 64^3 grid of
    amr64_f64.npz and on 256^3 grids of levels {2,3,4}, {1,2} and {3,4}
    (hashes in dump_ref.json, made by oracle/_ref/ref_dump_b16);
  * the refinement and compression plans reproduce the reference's forced
    regrid (Grid::refine, then Grid::compress) of amr64_f64.npz;
  * the whole adaptive time loop of Glioma_HG_UQ::run -- steps, regrids
    (one refinement pass, compression to a fixpoint) at the dump times --
    driven on the CPU with the AMR oracle's step, FWT and data movement and
    the library's plans and tables, ends on the reference's blocks and
    densities bit for bit, in FP64 and in the default FP32 build's
    arithmetic."""
import hashlib

import numpy as np
import pytest

from gliomauq_gb300 import _lib, amr, synthetic as S
from helpers import golden_json, golden_npz
from oracle import amr_oracle as A

REAL = {"f64": np.float64, "f32": np.float32}


def tables_sha(tables):
    st, sb, sc, w = tables
    h = hashlib.sha256()
    for a, t in ((st, "<i8"), (sb, "<i4"), (sc, "<i4"), (w, "<f8")):
        h.update(np.ascontiguousarray(a, dtype=t).tobytes())
    return h.hexdigest()


def test_ghost_tables_match_reference_on_the_adaptive_64_grid(gbg):
    d = golden_npz("amr64_f64.npz")
    st, sb, sc, w = _lib.amr_ghost_tables(d["blocks"])
    assert np.array_equal(st, d["ghost_start"])
    assert np.array_equal(sb, d["ghost_src_block"])
    assert np.array_equal(sc, d["ghost_src_cell"].astype(np.int32))
    assert np.array_equal(w, d["ghost_w"].astype(np.float64))


@pytest.mark.parametrize("name", ["grid3", "grid12", "grid34"])
def test_ghost_tables_match_reference_on_256_grids(gbg, name):
    ref = golden_json("dump_ref.json")[name]
    bl = np.array(ref["blocks"], dtype=np.int32)
    t = _lib.amr_ghost_tables(bl)
    assert len(t[1]) == ref["table_entries"]
    assert tables_sha(t) == ref["tables_sha256"]


def test_ghost_tables_reject_a_grid_that_is_not_a_tree(gbg):
    blocks = np.array(amr.uniform_blocks(1))
    with pytest.raises(_lib.GbgError):
        _lib.amr_ghost_tables(blocks[:-1])  # a hole
    bad = blocks.copy()
    bad[0] = (0, 0, 0, 0)                   # overlaps the others
    with pytest.raises(_lib.GbgError):
        _lib.amr_ghost_tables(bad)


def test_plans_reproduce_the_reference_forced_regrid(gbg):
    """ref_harness state's forced regrid: Grid::refine of every block below
    the maximum level 2 (the refiner adds what its rules add), then
    Grid::compress offered every block that existed before and lies in the
    upper half of x."""
    d = golden_npz("amr64_f64.npz")
    b0 = d["blocks"]
    nb1, k1, _, nref = _lib.amr_plan_refine(b0, (b0[:, 0] < 2).astype(np.uint8), max_level=2)
    assert nref == int((b0[:, 0] < 2).sum())
    offer = (k1 == 0) & (nb1[:, 1] >= (1 << nb1[:, 0]) // 2)
    nb2, k2, src, ncol = _lib.amr_plan_compress(nb1, offer.astype(np.uint8))
    assert ncol >= 1 and set(k2.tolist()) >= {0, 2}
    assert set(map(tuple, nb2.tolist())) == set(map(tuple, d["s2_blocks"].tolist()))


def test_refine_plan_keeps_level_jumps_at_one_across_periodic_faces(gbg):
    """Refining one block of a level-1 grid at a domain corner: its
    neighbours through the periodic faces are at most one level coarser than
    its children, and nothing above the maximum level is made."""
    blocks = np.array(amr.uniform_blocks(1))
    flag = np.zeros(len(blocks), np.uint8)
    flag[0] = 1
    nb1, kind, src, n = _lib.amr_plan_refine(blocks, flag, max_level=3)
    assert n == 1 and len(nb1) == 7 + 8
    flag = (np.arange(len(nb1)) == int(np.argmax(kind == 1))).astype(np.uint8)
    nb2, _, _, n2 = _lib.amr_plan_refine(nb1, flag, max_level=3)
    # refining a level-2 child to 3: the level-1 blocks next to it are two
    # levels coarser than its children, so the jump rule refines them too
    # (and the space extension refines every level-1 block touching a
    # level-2 one)
    lv = nb2[:, 0]
    assert lv.max() == 3 and (lv == 1).sum() == 0 and n2 == 8
    assert len(nb2) == 7 + 7 * 8 + 8
    st, _, _, _ = _lib.amr_ghost_tables(nb2)  # a valid tree with jumps <= 1
    assert st.size == len(nb2) * 1736 + 1


def oracle_adaptive_run(blocks, pw, pg, phi, Dw_file, rho, tend, L, bpd, dumpfreq, max_level,
                        real, final_refine=False, refine_tol=1e-4, compress_tol=1e-5):
    """Glioma_HG_UQ::run (Glioma_HG_UQ.cpp:511-582) on the CPU: the AMR
    oracle's step, FWT and data movement, the library's host-only tables and
    plans. Returns (blocks, phi, steps, regrids)."""
    f32 = real is np.float32
    dt, dw, dg = S.reference_dt(16 * bpd, Dw_file, L, f32=f32)
    if f32:
        rho = float(np.float32(rho))
    blocks = np.asarray(blocks, dtype=np.int32)
    pw, pg, phi = (np.asarray(x, dtype=real).reshape(-1, 4096) for x in (pw, pg, phi))
    tables = _lib.amr_ghost_tables(blocks)

    def move(new_blocks, kind, src):
        nonlocal blocks, pw, pg, phi, tables
        out = []
        for f in (pw, pg, phi):
            g = A.ghost_values(f, *tables[:3], tables[3], real)
            out.append(A.remap(f, g, kind, src, real).reshape(-1, 4096))
        pw, pg, phi = out
        blocks = np.asarray(new_blocks, dtype=np.int32)
        tables = _lib.amr_ghost_tables(blocks)

    def refine():
        cand = blocks[:, 0] < max_level
        if not cand.any():
            return
        det = A.fwt_detail(phi, tables, real)
        flag = cand & (det >= refine_tol)
        if flag.any():
            nb, kind, src, _ = _lib.amr_plan_refine(blocks, flag.astype(np.uint8), max_level)
            move(nb, kind, src)

    def compress():
        nice = set()
        while True:
            keys = [tuple(b) for b in blocks.tolist()]
            cand = np.array([k not in nice for k in keys])
            if not cand.any():
                return
            det = A.fwt_detail(phi, tables, real)
            flag = cand & (det < compress_tol)
            nice |= {k for k, c, f in zip(keys, cand, flag) if c and not f}
            if not flag.any():
                return
            nb, kind, src, n = _lib.amr_plan_compress(blocks, flag.astype(np.uint8))
            if n == 0:
                return
            move(nb, kind, src)

    t, when, steps, regrids = 0.0, dumpfreq, 0, 0
    while t <= tend:
        phi = A.step(blocks[:, 0], pw, pg, phi, tables, dw, dg, rho, dt, real).reshape(-1, 4096)
        t += dt
        steps += 1
        if t >= when:
            refine()
            compress()
            regrids += 1
            when = when + dumpfreq
    if final_refine:
        refine()
        regrids += 1
    return blocks, phi, steps, regrids


@pytest.mark.parametrize("variant", ["f64", "f32"])
def test_adaptive_loop_on_cpu_matches_reference(gbg, variant):
    """The input of amr64_*.npz (64^3 anatomy, Gaussian bump, Dw 0.0013,
    rho 0.1, T 60, regrid every 25 days, 4^3 blocks at the maximum level 2):
    after the loop the grid and every density equal the reference's."""
    d = golden_npz(f"amr64_{variant}.npz")
    a = golden_npz("anatomy64.npz")
    pw, pg = a["p_w"].astype(np.float64), a["p_g"].astype(np.float64)
    an = S.Anatomy(n=64, p_w=pw, p_g=pg, psi=None)
    phi0 = S.gaussian_ic(an, 20.3, 24.6, 22.1, peak=0.5, sigma=1.5).astype(np.float32)
    bl0 = amr.uniform_blocks(2)
    blocks, phi, steps, regrids = oracle_adaptive_run(
        bl0, amr.to_block_major(pw, 2), amr.to_block_major(pg, 2),
        amr.to_block_major(phi0.astype(np.float64), 2), 0.0013, 0.1, 60.0, 6.4, 4, 25.0, 2,
        REAL[variant])
    assert regrids == 2
    ref = {tuple(b): i for i, b in enumerate(d["blocks"].tolist())}
    assert set(map(tuple, blocks.tolist())) == set(ref), "block structure differs"
    for i, b in enumerate(blocks.tolist()):
        got = phi[i].astype(np.float64).reshape(16, 16, 16)
        assert np.array_equal(got, d["phi"][ref[tuple(b)]]), b


@pytest.mark.parametrize("variant", ["f64", "f32"])
def test_long_adaptive_run_on_cpu_matches_reference(gbg, variant):
    """tests/golden/adaptive64.json: the reference's run with a regrid every
    10 days to 110 days and the final refinement (refinements, including the
    space extension, and compressions both occur): same step and regrid
    counts, same final blocks, densities bit for bit (hash)."""
    import sys
    import os
    sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
    from make_golden import ADAPTIVE64 as c, adaptive_phi_sha
    ref = golden_json("adaptive64.json")[variant]
    a = golden_npz("anatomy64.npz")
    pw, pg = a["p_w"].astype(np.float64), a["p_g"].astype(np.float64)
    an = S.Anatomy(n=64, p_w=pw, p_g=pg, psi=None)
    phi0 = S.gaussian_ic(an, *c["seed_xyz"], peak=c["peak"], sigma=c["sigma"]).astype(np.float32)
    blocks, phi, steps, regrids = oracle_adaptive_run(
        amr.uniform_blocks(2), amr.to_block_major(pw, 2), amr.to_block_major(pg, 2),
        amr.to_block_major(phi0.astype(np.float64), 2), c["Dw"], c["rho"], c["tend"], c["L"],
        c["bpd"], c["dumpfreq"], c["max_level"], REAL[variant], final_refine=True)
    assert (steps, regrids) == (ref["steps"], ref["regrids"])
    assert sorted(blocks.tolist()) == ref["blocks"]
    assert adaptive_phi_sha(blocks.tolist(), phi.astype(np.float64)) == ref["phi_sha256"]
