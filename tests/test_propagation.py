"""CPU: the oracle's restatement of the reference's posterior propagation
statistics (per-cell mean and variance over the samples' final densities,
source/Glioma/Glioma_HG_Propagation.cpp:346-440) against the reference
program's own outputs on seeded fields (tests/golden/propagation.json, made by
make_golden.py propagation)."""
import os
import sys

import numpy as np
import pytest

from helpers import golden_json

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
from make_golden import PROPAGATION, propagation_fields, sha  # noqa: E402


@pytest.mark.parametrize("case", range(len(PROPAGATION)))
def test_oracle_statistics_equal_reference_program(case, oracle_lib):
    ref = golden_json("propagation.json")[case]
    c = PROPAGATION[case]
    assert {k: ref[k] for k in c} == c
    fields = propagation_fields(c["n"], c["S"], c["seed"])
    mean, var = oracle_lib.propagation_stats(fields)
    assert sha(mean) == ref["mean_sha256"]
    assert sha(var) == ref["var_sha256"]


def test_oracle_statistics_without_index_rule(oracle_lib):
    """reference_rules = False fills the zero-index planes with the same
    arithmetic; the interior is unchanged and matches float64 moments to
    float32 rounding."""
    fields = propagation_fields(16, 5, 3)
    m0, v0 = oracle_lib.propagation_stats(fields)
    m1, v1 = oracle_lib.propagation_stats(fields, reference_rules=False)
    assert np.array_equal(m0[1:, 1:, 1:], m1[1:, 1:, 1:])
    assert np.array_equal(v0[1:, 1:, 1:], v1[1:, 1:, 1:])
    assert not np.any(m0[0]) and np.any(m1[0])
    F = fields.astype(np.float64)
    assert np.allclose(m1, F.mean(0), rtol=0, atol=1e-6)
    assert np.allclose(v1, F.var(0), rtol=0, atol=1e-6)
