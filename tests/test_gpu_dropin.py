"""GPU: the C++ drop-in back-end (include/gbglioma_blockprocessing.hpp) run at
the reference's call-site shape on a mock MRAG grid:
* uniform grid: the fused GPU steps equal the C-ABI step bitwise, an unknown
  functor falls back to the CPU back-end on current host data, and the GPU
  state is re-uploaded after it;
* mixed-level grid: the steps equal the reference's own steps on that grid
  (amr64_f64.npz, made by the reference's MRAG pipeline) bit for bit;
* HostSync::at_times: the host blocks at the run loop's output times and at
  its end equal those of HostSync::every_step, with far fewer copies;
* the per-step cost of both modes at 128^3."""
import os
import subprocess

import numpy as np
import pytest

from gliomauq_gb300 import _lib, amr
from helpers import golden_npz

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def exe(gbg, tmp_path_factory):
    out = str(tmp_path_factory.mktemp("dropin") / "dropin_mock_run")
    libdir = os.path.join(ROOT, "gliomauq_gb300")
    subprocess.run(["g++", "-O2", "-std=c++14", "-I" + os.path.join(ROOT, "include"),
                    "-I" + os.path.join(ROOT, "tests", "cpp"),
                    os.path.join(ROOT, "tests", "cpp", "dropin_mock_run.cpp"), "-o", out,
                    "-L" + libdir, "-lgbglioma", "-Wl,-rpath," + libdir], check=True)
    return out


def _grid_text(blocks, pw, pg, phi):
    lines = [str(len(blocks))] + [" ".join(str(int(v)) for v in b) for b in blocks]
    lines += [repr(float(v)) for a in (pw, pg, phi) for v in np.asarray(a).ravel()]
    return "\n".join(lines) + "\n"


def _run(exe, args, text):
    p = subprocess.run([exe] + [str(a) for a in args], input=text, capture_output=True, text=True,
                       check=True)
    return p


def _uniform32():
    d = golden_npz("rd32.npz")
    pw, pg, phi0 = (d[k].astype(np.float64) for k in ("p_w", "p_g", "phi0"))
    prm = tuple(float(d[k]) for k in ("Dw_f64", "Dg_f64", "rho", "dt_f64"))
    return pw, pg, phi0, prm


def test_dropin_uniform_grid_and_cpu_fallback(exe):
    pw, pg, phi0, (Dw, Dg, rho, dt) = _uniform32()
    text = _grid_text(amr.uniform_blocks(1), amr.to_block_major(pw, 1), amr.to_block_major(pg, 1),
                      amr.to_block_major(phi0, 1))
    p = _run(exe, [repr(Dw), repr(Dg), repr(rho), repr(dt)], text)
    assert "gpu_steps=8 cpu_calls=1 uploads=2" in p.stderr
    out = amr.from_block_major(np.array([float(x) for x in p.stdout.split()]).reshape(-1, 4096), 1)
    with _lib.Handle(32, "f64") as h:
        h.set_anatomy(pw, pg)
        h.set_phi(phi0)
        h.rd_step(Dw, Dg, rho, dt, 5)
        h.set_phi(h.get_phi() * 2.0)
        h.rd_step(Dw, Dg, rho, dt, 3)
        exp = h.get_phi()
    assert np.array_equal(out, exp)


def test_dropin_mixed_level_grid_equals_reference(exe):
    d = golden_npz("amr64_f64.npz")
    text = _grid_text(d["blocks"], d["p_w"], d["p_g"], d["phi"])
    p = _run(exe, [repr(float(d["Dw"])), repr(float(d["Dg"])), repr(float(d["rho"])),
                   repr(float(d["dt"])), "steps", int(d["steps_after"])], text)
    out = np.array([float(x) for x in p.stdout.split()]).reshape(-1, 4096)
    assert np.array_equal(out, d["phi_after"].reshape(-1, 4096))


def test_dropin_host_sync_at_the_run_loops_output_times(exe):
    pw, pg, phi0, (Dw, Dg, rho, dt) = _uniform32()
    text = _grid_text(amr.uniform_blocks(1), amr.to_block_major(pw, 1), amr.to_block_major(pg, 1),
                      amr.to_block_major(phi0, 1))
    p = _run(exe, [repr(Dw), repr(Dg), repr(rho), repr(dt), "schedule"], text)
    line = p.stdout.strip()
    assert line.startswith("schedule ok"), line
    syncs = int(line.split("syncs=")[1].split()[0])
    outputs = int(line.split("outputs=")[1])
    assert syncs <= outputs < 10  # 10 steps; one copy per output time at most


def test_dropin_step_cost_at_128(exe):
    pw, pg, phi0, (Dw, Dg, rho, dt) = _uniform32()
    text = _grid_text(amr.uniform_blocks(1), amr.to_block_major(pw, 1), amr.to_block_major(pg, 1),
                      amr.to_block_major(phi0, 1))
    p = _run(exe, [repr(Dw), repr(Dg), repr(rho), repr(dt), "time", 8, 50], text)
    print(p.stdout)
    ms = {l.split()[0]: float(l.split()[1]) for l in p.stdout.strip().splitlines()}
    assert ms["at_times"] < ms["every_step"]
