"""CPU: the drop-in back-end (include/gbglioma_blockprocessing.hpp) wired
into the reference's own Grid, BlockCollection, BoundaryInfo and Glioma
operators (compiled in place from the reference sources), with the library
replaced by a CPU stand-in (tests/cpp/gbg_amr_cpu_stub.cpp, steps computed
by the oracle's C restatement): through Glioma_HG_UQ's
_reactionDiffusionStep body it gives the same grid as the reference's own
block-processing pipeline, bit for bit, in the float and the double build;
an unknown functor runs on the reference's pipeline after a host sync; and
with HostSync::at_times the host blocks are current at every output time
of the run loop and at its end, with one read-back per output time."""
import os
import subprocess

import pytest

from oracle import refio

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module", params=["float", "double"])
def exe(request, tmp_path_factory, oracle_lib):
    if not os.path.isdir(refio.REF_SOURCE):
        pytest.skip("reference tree not present")
    ref = refio.REF_SOURCE
    out = str(tmp_path_factory.mktemp("wiring") / f"dropin_reference_run_{request.param}")
    odir = os.path.join(ROOT, "oracle")
    subprocess.run(["g++", "-O2", "-std=gnu++11", "-fpermissive", "-w", "-ffp-contract=off", "-fopenmp",
                    f"-D_MRAG_REAL_={request.param}", "-I" + os.path.join(odir, "shim"),
                    "-I" + os.path.join(odir, "shim", "vtk"), "-I" + ref, "-I" + os.path.join(ref, "Glioma"),
                    "-I" + os.path.join(ROOT, "include"), "-I" + odir,
                    os.path.join(ROOT, "tests", "cpp", "dropin_reference_run.cpp"),
                    os.path.join(ROOT, "tests", "cpp", "gbg_amr_cpu_stub.cpp"),
                    os.path.join(ref, "MRAGcore", "MRAGBoundaryBlockInfo.cpp"),
                    os.path.join(ref, "MRAGcore", "MRAGWavelets_StaticData.cpp"),
                    os.path.join(ref, "MRAGcore", "MRAGProfiler.cpp"), "-o", out, "-L" + odir, "-loracle",
                    "-Wl,-rpath," + odir, "-lpthread"], check=True)
    return out, request.param


def test_dropin_steps_the_reference_grid_like_its_own_pipeline(exe):
    path, real = exe
    p = subprocess.run([path], capture_output=True, text=True)
    print(p.stdout)
    assert p.returncode == 0, p.stdout + p.stderr
    line = p.stdout.strip().splitlines()[-1]
    assert line.startswith("equal 32768 diff=0")
    # 10 fused steps; uploads at the first step and after the CPU functor;
    # every_step reads phi back after each step
    assert "steps=10 uploads=2 calls=2,2,10,10" in line
    assert f"real={4 if real == 'float' else 8}" in line


def test_dropin_host_sync_at_the_run_loops_output_times_on_the_reference_grid(exe):
    path, _ = exe
    p = subprocess.run([path, "schedule"], capture_output=True, text=True)
    print(p.stdout)
    assert p.returncode == 0, p.stdout + p.stderr
    line = p.stdout.strip().splitlines()[-1]
    assert line.startswith("schedule ok outputs=4 syncs=4 steps=10")
