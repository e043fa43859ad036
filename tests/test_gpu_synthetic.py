"""GPU: synthetic observations (gbg_synthetic_observations and gbg_brain
-anatomy syntheticData) against the reference's own synthetic-data program
(Glioma_ProcessSyntheticData, golden hashes in tests/golden/synthetic.json):
PET, T1, T2 and the centre of mass bit for bit in the program's block loop
order, the oracle's in x-fastest order, and the error cases."""
import os
import subprocess
import sys

import numpy as np
import pytest

from gliomauq_gb300 import _lib, build, matrix_io
from helpers import GOLDEN, golden_json

pytestmark = pytest.mark.gpu
sys.path.insert(0, GOLDEN)
from make_golden import SYNTHETIC, sha, synthetic_tumour  # noqa: E402


@pytest.mark.parametrize("case", range(len(SYNTHETIC)))
def test_synthetic_observations_equal_reference_program(gbg, case):
    ref = golden_json("synthetic.json")[case]
    c = SYNTHETIC[case]
    u = synthetic_tumour(c["n"], c["centre"], c["radius"])
    pet, t1, t2, com = _lib.synthetic_observations(u, ref["block_order"])
    assert sha(t1) == ref["t1_sha256"] and sha(t2) == ref["t2_sha256"]
    assert sha(pet) == ref["pet_sha256"]
    assert [float(v) for v in com] == ref["centre_of_mass"]


def test_synthetic_observations_default_order_equals_oracle(gbg, oracle_lib):
    c = SYNTHETIC[0]
    u = synthetic_tumour(c["n"], c["centre"], c["radius"])
    pet, t1, t2, com = _lib.synthetic_observations(u)
    n = c["n"] // 16
    xfast = [(2, x, y, z) for z in range(n) for y in range(n) for x in range(n)]
    op, o1, o2, ocom = oracle_lib.synthetic_observations(u, xfast)
    assert np.array_equal(t1, o1) and np.array_equal(t2, o2)
    diff = np.flatnonzero(pet != op)
    print("cells differing from the oracle:", diff.size)
    assert diff.size == 0
    assert np.array_equal(com, ocom)


def test_synthetic_observations_errors(gbg):
    u = np.zeros((32, 32, 32))
    with pytest.raises(_lib.GbgError):
        _lib.synthetic_observations(u)  # no cell reaches the threshold
    u[10, 10, 10] = 0.9
    with pytest.raises(_lib.GbgError):
        _lib.synthetic_observations(u, [(1, 0, 0, 0)] * 8)  # not a permutation
    with pytest.raises(_lib.GbgError):
        _lib.synthetic_observations(np.zeros((24, 24, 24)))  # n not 16 * 2^l
    pet, t1, t2, com = _lib.synthetic_observations(u)
    assert pet.max() == 1.0 and t1.sum() == 1 and t2.sum() == 1


def test_brain_synthetic_data_equals_reference_program(gbg, tmp_path):
    cli = dict(zip(build.CLI_PROGRAMS, build.build_cli()))
    ref = golden_json("synthetic.json")[0]
    c = SYNTHETIC[0]
    matrix_io.write_d3d(str(tmp_path / "HGG_data.dat"), synthetic_tumour(c["n"], c["centre"], c["radius"]))
    np.savetxt(str(tmp_path / "order.txt"), np.array(ref["block_order"]), fmt="%d")
    subprocess.run([cli["gbg_brain"], "-anatomy", "syntheticData", "-adaptive", "0", "-vtk", "0",
                    "-verbose", "0", "-blockorder", "order.txt"], cwd=tmp_path, check=True)
    for k in ("PET", "T1", "T2"):
        assert sha(matrix_io.read_d3d(str(tmp_path / f"{k}_data.dat"))) == ref[f"{k.lower()}_sha256"], k
    com = np.fromfile(str(tmp_path / "HGG_TumorIC.bin"), dtype="<f4")
    assert com.size == 3 and [float(v) for v in com] == ref["centre_of_mass"]
