"""CPU: the oracle's restatement of the reference's synthetic-data processing
(source/Glioma/Glioma_ProcessSyntheticData.cpp: thresholds, PET statistics,
drand48 noise through Box-Muller, normalisations) against the reference
program's own outputs on seeded tumours (tests/golden/synthetic.json, made
by make_golden.py synthetic): PET, T1, T2 and the centre of mass bit for
bit."""
import os
import sys

import numpy as np
import pytest

from helpers import golden_json

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
from make_golden import SYNTHETIC, sha, synthetic_tumour  # noqa: E402


@pytest.mark.parametrize("case", range(len(SYNTHETIC)))
def test_oracle_synthetic_data_equals_reference_program(case, oracle_lib):
    ref = golden_json("synthetic.json")[case]
    c = SYNTHETIC[case]
    u = synthetic_tumour(c["n"], c["centre"], c["radius"])
    pet, t1, t2, com = oracle_lib.synthetic_observations(u, ref["block_order"])
    assert int((pet > 0).sum()) <= ref["tumour_cells"]
    assert sha(pet) == ref["pet_sha256"]
    assert sha(t1) == ref["t1_sha256"]
    assert sha(t2) == ref["t2_sha256"]
    assert [float(v) for v in com] == ref["centre_of_mass"]


def test_oracle_noise_depends_on_the_block_order(oracle_lib):
    """The noise a cell receives follows the grid's loop order (the
    reference's comes from MRAG's node map, ordered by node address): the
    same tumour in x-fastest block order gives other PET values, the same
    thresholds, and a centre of mass within float rounding of noise."""
    ref = golden_json("synthetic.json")[1]
    c = SYNTHETIC[1]
    u = synthetic_tumour(c["n"], c["centre"], c["radius"])
    xfast = [(1, x, y, z) for z in range(2) for y in range(2) for x in range(2)]
    assert xfast != ref["block_order"]
    pet, t1, t2, com = oracle_lib.synthetic_observations(u, xfast)
    assert sha(pet) != ref["pet_sha256"]
    assert sha(t1) == ref["t1_sha256"] and sha(t2) == ref["t2_sha256"]
    assert np.allclose(com, ref["centre_of_mass"], atol=2e-3)
