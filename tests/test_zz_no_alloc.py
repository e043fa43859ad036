"""GPU: gbg_loglik_noalloc, the log-likelihood entry point that allocates
nothing (for callers that cannot call cudaMalloc: hosts whose device memory
belongs to another allocator, fixed real-time budgets). Called through the C ABI twice in a row, each result must
match the handle-based gbg_loglik on the same field and observations, and the
CPU oracle (pinned to the reference's likelihood program), which shares no
code with the two GPU entry points.

This file is named to be collected last, so a run that stops at the first
failure has already run every other test."""
import ctypes as C

import numpy as np
import pytest

from gliomauq_gb300 import _lib
from helpers import golden_json, golden_npz

pytestmark = pytest.mark.gpu

REL_TOL = 1e-11  # the tolerance of the other likelihood tests


def compact_lists(n, pet, t1, t2, points, step_pet, step_ti):
    """The observation lists gbg_set_observations builds (same traversal)."""
    z, y, x = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    keep = (x % step_pet == 0) & (y % step_pet == 0) & (z % step_pet == 0) & (pet > 0)
    pet_idx = np.flatnonzero(keep.ravel()).astype(np.int32)
    pet_val = pet.ravel()[pet_idx].astype(np.float64)
    p = np.asarray(points, dtype=np.int64)
    sel = (p[:, 0] % step_ti == 0) & (p[:, 1] % step_ti == 0) & (p[:, 2] % step_ti == 0)
    p = p[sel]
    ti_idx = (p[:, 0] + n * (p[:, 1] + n * p[:, 2])).astype(np.int32)
    return (pet_idx, pet_val, ti_idx, t1.ravel()[ti_idx].astype(np.float64),
            t2.ravel()[ti_idx].astype(np.float64))


def test_loglik_noalloc_matches_handle_entry_twice(gbg, oracle_lib):
    torch = pytest.importorskip("torch")
    d = golden_npz("lik32.npz")
    ref = golden_json("lik32.json")
    n, sp, st = 32, 3, 2
    pet, t1, t2 = (d[k].astype(np.float64) for k in ("pet", "t1", "t2"))
    fields = [d["model"].astype(np.float32),
              np.roll(d["model"], 2, axis=1).astype(np.float32)]
    lists = compact_lists(n, pet, t1, t2, d["points"], sp, st)
    dev = torch.device("cuda:0")
    tl = [torch.from_numpy(np.ascontiguousarray(a)).to(dev) for a in lists]
    params = _lib.LikParams(*ref["params"], sp, st, 1)
    out = torch.zeros(5, dtype=torch.float64, device=dev)  # one gbg_lik_result
    stream = torch.cuda.current_stream(dev).cuda_stream
    for field in fields:
        with _lib.Handle(n, "f32") as h:
            h.set_phi(field.astype(np.float64))
            h.set_observations(pet, t1, t2, d["points"], ref["params"], step_pet=sp,
                               step_ti=st, selective=True)
            exp = h.loglik()
        phi = torch.from_numpy(field).to(dev)
        torch.cuda.synchronize()
        rc = gbg.gbg_loglik_noalloc(
            C.c_void_p(phi.data_ptr()), n, C.c_void_p(tl[0].data_ptr()),
            C.c_void_p(tl[1].data_ptr()), len(lists[0]), C.c_void_p(tl[2].data_ptr()),
            C.c_void_p(tl[3].data_ptr()), C.c_void_p(tl[4].data_ptr()), len(lists[2]),
            C.byref(params), C.c_void_p(out.data_ptr()), C.c_void_p(stream))
        assert rc == 0, gbg.gbg_last_error()
        torch.cuda.synchronize()
        raw = out.cpu().numpy()
        got = dict(l_pet=raw[0], l_t1=raw[1], l_t2=raw[2], total=raw[3],
                   n_pet=int(raw[4:5].view(np.int64)[0]))
        assert got["n_pet"] == exp["n_pet"]
        o = oracle_lib.loglik(field.astype(np.float64), pet, t1, t2, d["points"], ref["params"],
                              step_pet=sp, step_ti=st, selective=True)
        assert got["n_pet"] == o["n_pet"]
        for k in ("l_pet", "l_t1", "l_t2", "total"):
            assert abs(got[k] - exp[k]) <= REL_TOL * max(1.0, abs(exp[k])), (k, got[k], exp[k])
            assert abs(got[k] - o[k]) <= REL_TOL * max(1.0, abs(o[k])), (k, got[k], o[k])


def test_loglik_noalloc_rejects_oversize_and_bad_args(gbg):
    torch = pytest.importorskip("torch")
    params = _lib.LikParams(0.0025, 1.0, 0.7, 0.25, 0.09, 3, 2, 1)
    buf = torch.zeros(8, dtype=torch.float64, device="cuda:0")
    b = C.c_void_p(buf.data_ptr())  # valid device memory; the size check fails before any launch
    too_many = 4096 * 2048 + 1
    rc = gbg.gbg_loglik_noalloc(b, 32, b, b, too_many, b, b, b, 1, C.byref(params), b, None)
    assert rc == -1 and b"GBG_NOALLOC_MAX_ENTRIES" in gbg.gbg_last_error()
    rc = gbg.gbg_loglik_noalloc(None, 32, None, None, 0, None, None, None, 0, C.byref(params),
                                None, None)
    assert rc == -1
