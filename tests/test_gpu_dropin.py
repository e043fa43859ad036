"""GPU: the C++ drop-in back-end (include/gbglioma_blockprocessing.hpp) run at
the reference's call-site shape on a mock MRAG grid: the fused GPU steps
equal the C-ABI step bitwise, an unknown functor falls back to the CPU
back-end on current host data, and the GPU state is re-uploaded after it."""
import os
import subprocess

import numpy as np
import pytest

from gliomauq_gb300 import _lib
from helpers import golden_npz

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_dropin_backend_on_mock_grid(gbg, tmp_path):
    exe = str(tmp_path / "dropin_mock_run")
    libdir = os.path.join(ROOT, "gliomauq_gb300")
    subprocess.run(["g++", "-O2", "-std=c++14", "-I" + os.path.join(ROOT, "include"),
                    "-I" + os.path.join(ROOT, "tests", "cpp"),
                    os.path.join(ROOT, "tests", "cpp", "dropin_mock_run.cpp"), "-o", exe,
                    "-L" + libdir, "-lgbglioma", "-Wl,-rpath," + libdir], check=True)
    d = golden_npz("rd32.npz")
    pw, pg, phi0 = (d[k].astype(np.float64) for k in ("p_w", "p_g", "phi0"))
    Dw, Dg, rho, dt = (float(d[k]) for k in ("Dw_f64", "Dg_f64", "rho", "dt_f64"))
    stdin = "\n".join(repr(float(v)) for a in (pw, pg, phi0) for v in a.ravel())
    p = subprocess.run([exe, repr(Dw), repr(Dg), repr(rho), repr(dt)], input=stdin,
                       capture_output=True, text=True, check=True)
    assert "gpu_steps=8 cpu_calls=1" in p.stderr
    out = np.array([float(x) for x in p.stdout.split()]).reshape(32, 32, 32)
    with _lib.Handle(32, "f64") as h:
        h.set_anatomy(pw, pg)
        h.set_phi(phi0)
        h.rd_step(Dw, Dg, rho, dt, 5)
        mid = h.get_phi() * 2.0
        h.set_phi(mid)
        h.rd_step(Dw, Dg, rho, dt, 3)
        exp = h.get_phi()
    assert np.array_equal(out, exp)
