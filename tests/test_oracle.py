"""CPU: the oracle restatement against the reference's own outputs (golden
fixtures made by tests/golden/make_golden.py from oracle/_ref) and host logic."""
import hashlib
import os

import numpy as np
import pytest

from gliomauq_gb300 import matrix_io, synthetic as S
from helpers import boundary_layer, golden_json, golden_npz
from oracle import refio


def _sha(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<f8").tobytes()).hexdigest()


@pytest.mark.parametrize("k", [1, 10, 60])
def test_oracle_f64_matches_reference_bitwise(oracle_lib, k):
    d = golden_npz("rd32.npz")
    pw, pg, phi0 = (d[x].astype(np.float64) for x in ("p_w", "p_g", "phi0"))
    out = oracle_lib.rd_solve(pw, pg, phi0, float(d["Dw_f64"]), float(d["Dg_f64"]),
                              float(d["rho"]), float(d["dt_f64"]), k, prec="f64")
    assert np.array_equal(out, d[f"phi_f64_{k}"])


@pytest.mark.parametrize("k", [1, 10, 60])
def test_oracle_f32ref_matches_reference_bitwise(oracle_lib, k):
    d = golden_npz("rd32.npz")
    pw, pg, phi0 = (d[x] for x in ("p_w", "p_g", "phi0"))
    out = oracle_lib.rd_solve(pw, pg, phi0, float(d["Dw_f32"]), float(d["Dg_f32"]),
                              float(d["rho"]), float(d["dt_f32"]), k, prec="f32ref")
    assert np.array_equal(out, d[f"phi_f32_{k}"])


@pytest.mark.parametrize("k", [1, 40])
@pytest.mark.parametrize("prec,variant", [("f64", "f64"), ("f32ref", "f32")])
def test_oracle_mala_matches_reference_bitwise(oracle_lib, prec, variant, k):
    """The MALA variant's step (phi and the slopes sRho, sD of
    Glioma_MALA_SlopesOperator.h) against the reference compiled in place."""
    d = golden_npz("mala32.npz")
    t = np.float64 if prec == "f64" else np.float32
    pw, pg, phi0 = (d[x].astype(t) for x in ("p_w", "p_g", "phi0"))
    phi, sr, sd = oracle_lib.mala_solve(pw, pg, phi0, float(d[f"Dw_{variant}"]),
                                        float(d[f"Dg_{variant}"]), float(d["rho"]),
                                        float(d[f"dt_{variant}"]), k, prec=prec)
    for name, a in (("phi", phi), ("sRho", sr), ("sD", sd)):
        g = d[f"{name}_{variant}_{k}"]
        assert np.array_equal(a, g), name
    # the slopes are not trivially zero
    assert np.abs(sr).max() > 0 and np.abs(sd).max() > 0


@pytest.mark.parametrize("variant", ["f64", "f32"])
def test_oracle_config1_full_solve(oracle_lib, variant):
    meta = golden_json("c1_64.json")
    a = golden_npz("anatomy64.npz")
    f32 = variant == "f32"
    dt, dw, dg = S.reference_dt(meta["n"], meta["Dw_file"], meta["L"], f32=f32)
    assert dt == meta[variant]["dt"]
    ns = S.num_steps(dt, meta["tend"])
    assert ns == meta[variant]["steps"] == 237
    out = oracle_lib.rd_solve(a["p_w"], a["p_g"], a["phi0"], dw, dg, meta["rho"], dt, ns,
                              prec="f32ref" if f32 else "f64")
    assert _sha(out.astype(np.float64)) == meta[variant]["sha256"]


def test_blocklab_port_matches_reference(oracle_lib):
    d = golden_npz("rd32.npz")
    g = oracle_lib.BlockGrid(d["p_w"], d["p_g"], d["phi0"])
    g.steps(float(d["Dw_f32"]), float(d["Dg_f32"]), float(d["rho"]), float(d["dt_f32"]), 10)
    assert np.array_equal(g.phi(), d["phi_f32_10"])


def test_boundary_layer_is_pinned_in_reference_output():
    d = golden_npz("rd32.npz")
    brain = (d["p_w"].astype(np.float64) + d["p_g"]) > 0
    layer = boundary_layer(brain)
    assert layer.sum() > 0
    for k in (1, 10, 60):
        u = d[f"phi_f64_{k}"]
        assert np.all(u[layer] == 0.0)
        assert np.all(u[~brain] == 0.0)
        assert not np.isnan(u).any()


@pytest.mark.parametrize("mode", ["sel", "all"])
def test_oracle_likelihood_matches_reference_program(oracle_lib, mode):
    d = golden_npz("lik32.npz")
    ref = golden_json("lik32.json")
    r = oracle_lib.loglik(d["model"], d["pet"], d["t1"], d["t2"], d["points"],
                          ref["params"], step_pet=ref["step_pet"], step_ti=ref["step_ti"],
                          selective=(mode == "sel"))
    exp = ref[mode]
    # the reference prints %Lf: six decimals
    assert r["n_pet"] == exp["n_pet"]
    assert abs(r["l_pet"] - exp["l_pet"]) <= 1e-6
    assert abs(r["l_t1"] - exp["l_t1"]) <= 1e-6
    assert abs(r["l_t2"] - exp["l_t2"]) <= 1e-6
    assert abs(-r["total"] - exp["minus_loglik"]) <= 1e-6


def test_num_steps_matches_oracle(oracle_lib):
    for dt, tend in [(1.2692307692307696, 300.0), (0.66, 100.0), (8.25, 500.0), (1.0, 3.0),
                     (0.1, 0.0), (1.0, -1.0)]:
        assert S.num_steps(dt, tend) == oracle_lib.lib().orc_num_steps(dt, tend)


def test_matrix_io_roundtrip_and_errors(tmp_path):
    a = np.random.default_rng(0).random((3, 4, 5))
    p = tmp_path / "a.dat"
    matrix_io.write_d3d(str(p), a)
    assert np.array_equal(matrix_io.read_d3d(str(p)), a)
    b = np.arange(12.0).reshape(3, 4)
    q = tmp_path / "b.dat"
    matrix_io.write_d2d(str(q), b)
    assert np.array_equal(matrix_io.read_d2d(str(q)), b)
    raw = bytearray(open(p, "rb").read())
    raw[0] = 0
    (tmp_path / "bad.dat").write_bytes(bytes(raw))
    with pytest.raises(matrix_io.MatrixFormatError):
        matrix_io.read_d3d(str(tmp_path / "bad.dat"))
    (tmp_path / "short.dat").write_bytes(open(p, "rb").read()[:40])
    with pytest.raises(matrix_io.MatrixFormatError):
        matrix_io.read_d3d(str(tmp_path / "short.dat"))
    with pytest.raises(matrix_io.MatrixFormatError):
        matrix_io.read_d2d(str(p))  # a 3-D file read as 2-D


def test_reference_sphere_file_format_reads():
    """The reference's own Sphere.dat (D2D<double> 80160 x 3) parses, when present."""
    path = os.path.join(refio.REF_SOURCE, "Likelihood", "makefile", "Sphere.dat")
    if not os.path.exists(path):
        pytest.skip("reference tree not present")
    m = matrix_io.read_d2d(path)
    assert m.shape == (3, 80160)
    assert m[0].min() >= 0 and m.max() < 128


@pytest.mark.skipif(not os.path.exists(os.path.join(os.path.dirname(__file__), "..", "oracle",
                                                    "_ref", "ref_harness_f64")),
                    reason="reference binaries not built here")
def test_oracle_live_vs_reference_random_case(oracle_lib):
    from oracle import refio
    rng = np.random.default_rng(123)
    n = 32
    an = S.make_anatomy(n, seed=77)
    pw = an.p_w.astype(np.float32).astype(np.float64)
    pg = an.p_g.astype(np.float32).astype(np.float64)
    phi0 = (rng.random((n, n, n)) * (pw + pg > 0)).astype(np.float32).astype(np.float64)
    Dw, rho = 0.002, 0.15
    r = refio.run_harness("solve", "f64", n, 2, pw, pg, phi0, Dw, rho, 0.0, n * 0.1, nsteps=5)
    out = oracle_lib.rd_solve(pw, pg, phi0, r["Dw"], r["Dg"], r["rho"], r["dt"], 5, prec="f64")
    assert np.array_equal(out, r["phi"])


@pytest.mark.skipif(not os.path.isdir(refio.REF_SOURCE), reason="reference tree not present")
def test_dropin_backend_compiles_against_reference_types():
    """include/gbglioma_blockprocessing.hpp instantiated at the reference's own
    call-site types (Grid, BlockCollection, BoundaryInfo, Glioma operators, the
    TBB pipeline as CPU back-end): a compile-only check."""
    import subprocess
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    ref = refio.REF_SOURCE
    r = subprocess.run(["g++", "-fsyntax-only", "-std=gnu++11", "-fpermissive", "-w",
                        "-I" + os.path.join(root, "oracle", "shim"),
                        "-I" + os.path.join(root, "oracle", "shim", "vtk"), "-I" + ref,
                        "-I" + os.path.join(ref, "Glioma"), "-I" + os.path.join(root, "include"),
                        os.path.join(root, "tests", "cpp", "dropin_reference_compile.cpp")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]


@pytest.mark.skipif(not os.path.exists(os.path.join(os.path.dirname(__file__), "..", "oracle",
                                                    "_ref", "brain")),
                    reason="reference binaries not built here")
def test_patient_initial_state_restatement_matches_reference_brain(tmp_path):
    """gbg_brain's restatement of _ic_PatientCase (cli/patient_ic.hpp) against
    the reference's own brain run with no time step (tend < 0)."""
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, os.path.join(root, "tests", "golden"))
    import make_golden
    from oracle import refio
    exe = str(tmp_path / "ic_dump")
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off",
                    "-I" + os.path.join(root, "gliomauq_gb300", "cli"),
                    os.path.join(root, "tests", "cpp", "patient_ic_dump.cpp"), "-o", exe], check=True)
    d = golden_npz("patient32.npz")
    pat = {k: d[k].astype(np.float64) for k in ("GM", "WM", "CSF", "T1", "T2")}
    pat["ic"] = [float(v) for v in d["ic"]]
    pat["params"] = [0.0013, 0.2, -1.0]
    work = make_golden.patient_files(str(tmp_path / "p"), pat)
    subprocess.run([os.path.join(refio.REF_DIR, "brain"), "-anatomy", "HGG_UQ", "-pID", "1",
                    "-adaptive", "0", "-dumpfreq", "1000", "-vtk", "0", "-verbose", "0",
                    "-nthreads", "1"], cwd=work, check=True, capture_output=True)
    ref = matrix_io.read_d3d(os.path.join(work, "HGG_data.dat"))
    out = str(tmp_path / "mine.dat")
    subprocess.run([exe, str(tmp_path / "p" / "Anatmoy" / "Patient01" / "P01"),
                    os.path.join(work, "HGG_TumorIC.bin"), out], check=True)
    assert np.array_equal(matrix_io.read_d3d(out), ref)
