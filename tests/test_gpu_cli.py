"""GPU: gbg_brain / gbg_likelihood against the reference's own `brain` and
`likelihood` programs (golden hashes from tests/golden/make_golden.py) on a
synthetic patient, through the same files and folder layout."""
import hashlib
import os
import subprocess
import sys

import numpy as np
import pytest

from gliomauq_gb300 import build, matrix_io
from helpers import GOLDEN, golden_json, golden_npz

pytestmark = pytest.mark.gpu
sys.path.insert(0, GOLDEN)
import make_golden  # noqa: E402  (fixture writers, no reference access at import)


def _sha(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<f8").tobytes()).hexdigest()


@pytest.fixture(scope="module")
def cli(gbg):
    return dict(zip(build.CLI_PROGRAMS, build.build_cli()))


def _patient(tmp_path, params):
    d = golden_npz("patient32.npz")
    pat = {k: d[k].astype(np.float64) for k in ("GM", "WM", "CSF", "T1", "T2")}
    pat["ic"] = [float(v) for v in d["ic"]]
    pat["params"] = params
    return make_golden.patient_files(str(tmp_path), pat)


def _brain(cli, work):
    subprocess.run([cli["gbg_brain"], "-anatomy", "HGG_UQ", "-pID", "1", "-adaptive", "0",
                    "-dumpfreq", "1000", "-vtk", "0", "-verbose", "0", "-nthreads", "1"],
                   cwd=work, check=True, capture_output=True)
    return matrix_io.read_d3d(os.path.join(work, "HGG_data.dat"))


def test_brain_initial_state_matches_reference(cli, tmp_path):
    ref = golden_json("patient32.json")
    work = _patient(tmp_path, [0.0013, 0.2, -1.0])
    u0 = _brain(cli, work)
    assert _sha(u0) == ref["brain_ic"]["sha256"]


def test_brain_and_likelihood_match_reference(cli, tmp_path):
    ref = golden_json("patient32.json")
    d = golden_npz("patient32.npz")
    work = _patient(tmp_path, [float(x) for x in d["params"]])
    u = _brain(cli, work)
    assert _sha(u) == ref["brain"]["sha256"]
    for k, v in make_golden.cli_observations(u).items():
        if k == "Sphere":
            matrix_io.write_d2d(os.path.join(work, "Sphere.dat"), v)
        else:
            matrix_io.write_d3d(os.path.join(work, f"{k}_data.dat"), v)
    with open(os.path.join(work, "LikelihoodInput.txt"), "w") as f:
        f.write("\n".join(repr(x) for x in make_golden.LIK_PARAMS) + "\n")
    subprocess.run([cli["gbg_likelihood"]], cwd=work, check=True, capture_output=True)
    got = float(open(os.path.join(work, "Likelihood.txt")).read().split()[0])
    assert abs(got - ref["likelihood"]) <= 2e-6


def test_adaptive_brain_matches_reference(cli, tmp_path):
    """gbg_brain -adaptive 1 (the library's block grid with its regrids)
    against the reference's brain built with _MAXLEVEL_ = 2, -adaptive 1
    -dumpfreq 10: HGG_data.dat bit for bit."""
    ref = golden_json("patient32.json")["brain_adaptive"]
    d = golden_npz("patient32.npz")
    work = _patient(tmp_path, [float(x) for x in d["params"]])
    subprocess.run([cli["gbg_brain"], "-anatomy", "HGG_UQ", "-pID", "1", "-adaptive", "1",
                    "-dumpfreq", "10", "-maxlevel", "2", "-vtk", "0", "-verbose", "0"],
                   cwd=work, check=True, capture_output=True)
    u = matrix_io.read_d3d(os.path.join(work, "HGG_data.dat"))
    assert _sha(u) == ref["sha256"]


def test_brain_rejects_bad_options_and_missing_files(cli, tmp_path):
    work = _patient(tmp_path, [0.0013, 0.2, 10.0])
    r = subprocess.run([cli["gbg_brain"], "-anatomy", "HGG_UQ", "-pID", "1", "-adaptive", "1",
                        "-maxlevel", "1"], cwd=work, capture_output=True, text=True)
    assert r.returncode != 0 and "maxlevel" in r.stderr
    r = subprocess.run([cli["gbg_brain"], "-anatomy", "HGG_UQ", "-pID", "1", "-bpd", "3"],
                       cwd=work, capture_output=True, text=True)
    assert r.returncode != 0 and "power of two" in r.stderr
    os.remove(os.path.join(work, "HGG_TumorIC.bin"))
    r = subprocess.run([cli["gbg_brain"], "-anatomy", "HGG_UQ", "-pID", "1"], cwd=work,
                       capture_output=True, text=True)
    assert r.returncode == 1 and "File error" in r.stderr
