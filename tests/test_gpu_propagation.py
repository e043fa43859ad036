"""GPU: posterior propagation statistics through the C ABI.
gbg_field_statistics on the seeded fields equals the reference's propagation
program bit for bit (tests/golden/propagation.json; the per-cell mean and
variance of source/Glioma/Glioma_HG_Propagation.cpp:346-440 in its float
Real); gbg_batch_statistics equals the oracle's statistics over the batched
solver's own final densities."""
import ctypes as C
import os
import sys

import numpy as np
import pytest

from gliomauq_gb300 import _lib, synthetic as S
from helpers import golden_json

pytestmark = pytest.mark.gpu

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
from make_golden import PROPAGATION, propagation_fields, sha  # noqa: E402


def _device_stats(gbg, fields, reference_rules):
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda:0")
    S_, n = fields.shape[0], fields.shape[1]
    f = torch.from_numpy(np.ascontiguousarray(fields)).to(dev)
    mean = torch.full((n, n, n), float("nan"), dtype=torch.float32, device=dev)
    var = torch.full((n, n, n), float("nan"), dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    rc = gbg.gbg_field_statistics(n, C.c_void_p(f.data_ptr()), S_, 1 if reference_rules else 0,
                                  C.c_void_p(mean.data_ptr()), C.c_void_p(var.data_ptr()),
                                  C.c_void_p(stream))
    assert rc == 0, gbg.gbg_last_error()
    torch.cuda.synchronize()
    return mean.cpu().numpy(), var.cpu().numpy()


@pytest.mark.parametrize("case", range(len(PROPAGATION)))
def test_field_statistics_equal_reference_program(gbg, case):
    ref = golden_json("propagation.json")[case]
    c = PROPAGATION[case]
    mean, var = _device_stats(gbg, propagation_fields(c["n"], c["S"], c["seed"]), True)
    assert sha(mean) == ref["mean_sha256"]
    assert sha(var) == ref["var_sha256"]


def test_field_statistics_without_index_rule_equal_oracle(gbg, oracle_lib):
    fields = propagation_fields(48, 7, 5)
    mean, var = _device_stats(gbg, fields, False)
    om, ov = oracle_lib.propagation_stats(fields, reference_rules=False)
    assert np.array_equal(mean, om)
    assert np.array_equal(var, ov)


@pytest.mark.parametrize("dt0", [0.0, -1.0])
def test_batch_statistics_equal_oracle_on_batch_fields(gbg, oracle_lib, dt0):
    """dt0 = 0: the reference's time loop; dt0 = -1: the stable scaled grid."""
    an = S.make_anatomy(32, seed=4)
    samples = [(0.0013, 0.025, 15.2, 16.1, 15.7, 60.0), (0.0025, 0.2, 14.0, 15.0, 16.0, 25.0),
               (0.0002, 0.01, 16.4, 16.6, 14.9, 130.0), (0.0009, 0.05, 15.0, 15.5, 16.5, 45.0),
               (0.0017, 0.12, 16.0, 14.5, 15.5, 80.0)]
    with _lib.Handle(32, "f32", max_samples=len(samples)) as h:
        h.set_anatomy(an.p_w, an.p_g)
        res = h.batch_solve(samples, an.L, with_loglik=False, want_phi=True, dt0=dt0)
        assert len(set(int(k) & 1 for k in res["nsteps"])) == 2  # both ping-pong buffers
        mean, var = h.batch_statistics(samples, an.L, dt0=dt0)
        mean2, var2 = h.batch_statistics(samples, an.L, dt0=dt0, reference_rules=False)
    om, ov = oracle_lib.propagation_stats(res["phi"])
    assert np.array_equal(mean, om.astype(np.float64))
    assert np.array_equal(var, ov.astype(np.float64))
    om, ov = oracle_lib.propagation_stats(res["phi"], reference_rules=False)
    assert np.array_equal(mean2, om.astype(np.float64))
    assert np.array_equal(var2, ov.astype(np.float64))
    assert var.max() > 0


def test_statistics_argument_errors(gbg):
    torch = pytest.importorskip("torch")
    buf = torch.zeros(8, dtype=torch.float32, device="cuda:0")
    b = C.c_void_p(buf.data_ptr())
    assert gbg.gbg_field_statistics(0, b, 1, 1, b, b, None) == -1
    assert gbg.gbg_field_statistics(8, b, 0, 1, b, b, None) == -1
    assert gbg.gbg_field_statistics(8, None, 1, 1, b, b, None) == -1
    with _lib.Handle(32, "f32", max_samples=2) as h:
        an = S.make_anatomy(32, seed=4)
        h.set_anatomy(an.p_w, an.p_g)
        with pytest.raises(_lib.GbgError):
            h.batch_statistics([(0.0013, 0.025, 15.2, 16.1, 15.7, 60.0)] * 3, an.L)
        with pytest.raises(_lib.GbgError):
            h.batch_statistics([(-1.0, 0.025, 15.2, 16.1, 15.7, 60.0)], an.L)
