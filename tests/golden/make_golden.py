"""Generates the golden fixtures in this folder from the reference itself.

Runs the GliomaUQ sources compiled in place by oracle/Makefile (oracle/_ref/:
the MRAG grid + TBB pipeline + Glioma operators through oracle/ref_harness.cpp,
and the reference's own `likelihood` program) on seeded synthetic inputs, and
stores inputs and outputs as small .npz/.json files. Inputs are rounded to
float32 values so that they are exact in both the FP32 and the FP64 build and
independent of the platform that regenerates them.

Usage (needs the reference's source tree at $GLIOMAUQ_REF, default
/root/reference/source, and `make -C oracle ref`):
    python tests/golden/make_golden.py
"""
from __future__ import annotations

import hashlib
import json
import os
import re
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from gliomauq_gb300 import matrix_io, synthetic as S  # noqa: E402
from oracle import refio  # noqa: E402

LIK_PARAMS = (0.0025, 1.0, 0.7, 0.25, 0.09)  # sigma2_PET, PETscale, T1uc, T2uc, slope


def f32(a):
    return np.asarray(a, dtype=np.float32).astype(np.float64)


def inputs(n, seed, seed_xyz):
    an = S.make_anatomy(n, seed=seed)
    pw, pg = f32(an.p_w), f32(an.p_g)
    an32 = S.Anatomy(n=n, p_w=pw, p_g=pg, psi=an.psi)
    phi0 = f32(S.gaussian_ic(an32, *seed_xyz))
    return pw, pg, phi0


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<f8").tobytes()).hexdigest()


def rd_fixtures():
    # 32^3 (2^3 blocks): snapshots after 1, 10 and 60 steps, FP64 and FP32 builds
    n, bpd = 32, 2
    pw, pg, phi0 = inputs(n, 3, (14.6, 16.3, 15.2))
    Dw, rho, L = 0.13 / 100, 0.025, n * 0.1
    out = dict(p_w=pw.astype(np.float32), p_g=pg.astype(np.float32),
               phi0=phi0.astype(np.float32), Dw_file=Dw, rho=rho, L=L)
    for variant in ("f64", "f32"):
        for k in (1, 10, 60):
            r = refio.run_harness("solve", variant, n, bpd, pw, pg, phi0, Dw, rho, 0.0, L, nsteps=k)
            out[f"phi_{variant}_{k}"] = r["phi"] if variant == "f64" else r["phi"].astype(np.float32)
            out[f"dt_{variant}"] = r["dt"]
            out[f"Dw_{variant}"] = r["Dw"]
            out[f"Dg_{variant}"] = r["Dg"]
    np.savez_compressed(os.path.join(HERE, "rd32.npz"), **out)

    # config 1: 64^3 (4^3 blocks), Dw = 0.13 mm^2/day, rho = 0.025/day, T = 300 days
    n, bpd = 64, 4
    pw, pg, phi0 = inputs(n, 1, (30.2, 33.7, 31.1))
    np.savez_compressed(os.path.join(HERE, "anatomy64.npz"), p_w=pw.astype(np.float32),
                        p_g=pg.astype(np.float32), phi0=phi0.astype(np.float32))
    meta = dict(n=n, Dw_file=0.13 / 100, rho=0.025, tend=300.0, L=n * 0.1)
    for variant in ("f64", "f32"):
        r = refio.run_harness("solve", variant, n, bpd, pw, pg, phi0, meta["Dw_file"], meta["rho"],
                              meta["tend"], meta["L"])
        u = r["phi"]
        meta[variant] = dict(steps=r["steps"], dt=r["dt"], sha256=sha(u), sum=float(u.sum()),
                             l2=float(np.linalg.norm(u)), max=float(u.max()))
        if variant == "f64":
            # a sparse sample of the field for readable failures
            rng = np.random.default_rng(0)
            idx = rng.choice(u.size, 256, replace=False)
            meta["sample_idx"] = idx.tolist()
            meta["sample_f64"] = u.ravel()[idx].tolist()
    with open(os.path.join(HERE, "c1_64.json"), "w") as f:
        json.dump(meta, f, indent=1)


def mala_fixture():
    # 32^3 (2^3 blocks): the MALA variant's step (phi and the slopes sRho, sD)
    # after 1 and 40 steps from zero slopes, FP64 and FP32 builds
    n, bpd = 32, 2
    pw, pg, phi0 = inputs(n, 3, (14.6, 16.3, 15.2))
    Dw, rho, L = 0.13 / 100, 0.025, n * 0.1
    out = dict(p_w=pw.astype(np.float32), p_g=pg.astype(np.float32),
               phi0=phi0.astype(np.float32), Dw_file=Dw, rho=rho, L=L)
    for variant in ("f64", "f32"):
        for k in (1, 40):
            r = refio.run_harness("mala", variant, n, bpd, pw, pg, phi0, Dw, rho, 0.0, L, nsteps=k)
            for f in ("phi", "sRho", "sD"):
                v = r[f]
                out[f"{f}_{variant}_{k}"] = v if variant == "f64" else v.astype(np.float32)
            out[f"dt_{variant}"] = r["dt"]
            out[f"Dw_{variant}"] = r["Dw"]
            out[f"Dg_{variant}"] = r["Dg"]
    np.savez_compressed(os.path.join(HERE, "mala32.npz"), **out)


def lik_fixture():
    """The reference `likelihood` program on a 32^3 model and seeded observations."""
    d = np.load(os.path.join(HERE, "rd32.npz"))
    model = d["phi_f64_60"]
    n = model.shape[0]
    an = S.Anatomy(n=n, p_w=d["p_w"].astype(np.float64), p_g=d["p_g"].astype(np.float64),
                   psi=None)
    # truth: the model itself a few steps later is not needed; use a shifted copy
    truth = np.roll(model, 1, axis=2)
    obs = S.make_observations(truth, an, seed=11, centre_xyz=(15.0, 16.0, 15.0), radius_vox=9.0)
    pet, t1, t2 = f32(obs.pet), obs.t1, obs.t2
    res = {}
    exe = os.path.join(refio.REF_DIR, "likelihood")
    for mode in ("sel", "all"):
        with tempfile.TemporaryDirectory() as td:
            matrix_io.write_d3d(os.path.join(td, "HGG_data.dat"), model)
            matrix_io.write_d3d(os.path.join(td, "PET_data.dat"), pet)
            matrix_io.write_d3d(os.path.join(td, "T1_data.dat"), t1)
            matrix_io.write_d3d(os.path.join(td, "T2_data.dat"), t2)
            matrix_io.write_d2d(os.path.join(td, "Sphere.dat"), obs.points.T)
            with open(os.path.join(td, "LikelihoodInput.txt"), "w") as f:
                f.write("\n".join(repr(x) for x in LIK_PARAMS) + "\n")
            args = [exe, "-selectivePoints", "1" if mode == "sel" else "0", "-stepPet", "2",
                    "-stepTi", "1"]
            p = subprocess.run(args, cwd=td, capture_output=True, text=True, check=True)
            m = re.search(r"L_Pet=([-\d.]+), L_T1=([-\d.]+), L_T2 = ([-\d.]+)", p.stdout)
            npet = int(re.search(r"Points=(\d+)", p.stdout).group(1))
            txt = float(open(os.path.join(td, "Likelihood.txt")).read().split()[0])
            res[mode] = dict(l_pet=float(m.group(1)), l_t1=float(m.group(2)),
                             l_t2=float(m.group(3)), minus_loglik=txt, n_pet=npet)
    np.savez_compressed(os.path.join(HERE, "lik32.npz"), model=model, pet=pet.astype(np.float32),
                        t1=t1.astype(np.uint8), t2=t2.astype(np.uint8),
                        points=obs.points.astype(np.int16))
    res.update(params=LIK_PARAMS, step_pet=2, step_ti=1)
    with open(os.path.join(HERE, "lik32.json"), "w") as f:
        json.dump(res, f, indent=1)


def region_starts():
    """Start of each of the 27 neighbour regions in a block's ghost list for
    the stencil [-1, 2) (region 13, the block itself, has none)."""
    out, start = [], 0
    for c in range(27):
        d = (c % 3 - 1, (c // 3) % 3 - 1, (c // 9) % 3 - 1)
        size = int(np.prod([16 if x == 0 else 1 for x in d]))
        out.append((start if c != 13 else 0, size if c != 13 else 0))
        if c != 13:
            start += size
    return out


def amr_fixtures():
    """Adaptive 64^3-effective grid (4^3 blocks at level 2, maximum level 2):
    the reference time loop with a regrid every 25 days to T = 60, then its
    blocks, ghost tables and FWT maxima, the blocks after 10 more steps, and
    the blocks after a forced regrid that splits and collapses (S2)."""
    a = np.load(os.path.join(HERE, "anatomy64.npz"))
    pw, pg = a["p_w"].astype(np.float64), a["p_g"].astype(np.float64)
    an = S.Anatomy(n=64, p_w=pw, p_g=pg, psi=None)
    phi0 = f32(S.gaussian_ic(an, 20.3, 24.6, 22.1, peak=0.5, sigma=1.5))
    for variant in ("f64", "f32"):
        st = refio.run_state(f"{variant}_l2", 64, 4, pw, pg, phi0, 0.0013, 0.1, 60.0, 6.4, 25.0,
                             extra=10)
        blocks = st["s0"]
        slot = {b["id"]: i for i, b in enumerate(blocks)}
        rs = region_starts()
        counts, sb, sc, w = [], [], [], []
        for g in st["ghosts"]:
            # region 13 is the block itself; MRAG leaves its record unset
            got = [tuple(r) for i, r in enumerate(g["regions"]) if i != 13]
            assert got == [r for i, r in enumerate(rs) if i != 13], "region layout differs"
            counts.append(g["counts"])
            sb.append(np.array([slot[x] for x in g["src_block"]], dtype=np.int32))
            sc.append(g["src_cell"])
            w.append(g["w"])
        counts = np.concatenate(counts)
        start = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
        assert [b["id"] for b in st["s1"]] == [b["id"] for b in blocks]
        np.savez_compressed(
            os.path.join(HERE, f"amr64_{variant}.npz"),
            blocks=np.array([[b["level"], *b["index"]] for b in blocks], dtype=np.int32),
            p_w=np.stack([b["p_w"] for b in blocks]), p_g=np.stack([b["p_g"] for b in blocks]),
            phi=np.stack([b["phi"] for b in blocks]), ghost_start=start,
            ghost_src_block=np.concatenate(sb), ghost_src_cell=np.concatenate(sc).astype(np.int16),
            ghost_w=np.concatenate(w).astype(np.float32), fwt=st["fwt"],
            phi_after=np.stack([b["phi"] for b in st["s1"]]), steps_after=10,
            dt=st["dt"], Dw=st["Dw"], Dg=st["Dg"], rho=st["rho"],
            s2_blocks=np.array([[b["level"], *b["index"]] for b in st["s2"]], dtype=np.int32),
            s2_phi=np.stack([b["phi"] for b in st["s2"]]),
            s2_p_w=np.stack([b["p_w"] for b in st["s2"]]),
            s2_p_g=np.stack([b["p_g"] for b in st["s2"]]))


def dump_fixtures():
    """The reference's own Glioma_HG_UQ::_dumpUQoutput (Glioma_HG_UQ.cpp:309-372)
    on multi-level grids, as SHA-256 of its HGG_data.dat:
      dump64 : the adaptive 64^3 grid of amr64_f64.npz (levels 1, 2; h = hf,
               2 hf), by ref_dump_b4 running the same loop;
      grid3  : a 256^3 grid of levels 2, 3, 4 (h = 4 hf, 2 hf, hf) made by
               ref_dump_b16 dumpgrid (two forced compressions), cell values
               refio.dumpgrid_phi;
      grid12 : a 256^3 grid of levels 1 and 2 (h = 8 hf, 4 hf): the dump
               replicates a level-1 cell 4^3 times where it covers 8^3 cells,
               and leaves the rest of the MatrixD3D it allocated with new[]
               uninitialised -- the hash covers the cells it writes;
      grid34 : a 256^3 grid of levels 3 and 4.
    For the 256^3 grids also the hash of the grid's ghost instruction tables
    (Grid::getBoundaryInfo, flattened in the grid's block order)."""
    a = np.load(os.path.join(HERE, "anatomy64.npz"))
    pw, pg = a["p_w"].astype(np.float64), a["p_g"].astype(np.float64)
    an = S.Anatomy(n=64, p_w=pw, p_g=pg, psi=None)
    phi0 = f32(S.gaussian_ic(an, 20.3, 24.6, 22.1, peak=0.5, sigma=1.5))
    r = refio.run_dump("ref_dump_b4", 64, 4, pw, pg, phi0, 0.0013, 0.1, 60.0, 6.4, dumpfreq=25.0)
    d = np.load(os.path.join(HERE, "amr64_f64.npz"))
    bl = np.array([[b["level"], *b["index"]] for b in r["blocks"]], dtype=np.int32)
    assert np.array_equal(bl, d["blocks"]), "the dump run's grid differs from amr64_f64"
    assert np.array_equal(np.stack([b["phi"] for b in r["blocks"]]), d["phi"])
    out = {"dump64": dict(gpd=64, sha256=sha(r["dump"]), nonzero=int(np.count_nonzero(r["dump"])))}
    for name, radii in (("grid3", [0.2, 0.45]), ("grid12", [0.0, 0.0, 0.4]), ("grid34", [0.35])):
        g = refio.run_dumpgrid("ref_dump_b16", radii)
        blocks = g["blocks"]
        th = hashlib.sha256()
        for arr, t in zip(g["tables"], ("<i8", "<i4", "<i4", "<f8")):
            th.update(np.ascontiguousarray(arr, dtype=t).tobytes())
        from oracle import amr_oracle as A
        written = A.dump_uniform(blocks, np.ones((len(blocks), 16, 16, 16)), g["gpd"]) != 0
        out[name] = dict(gpd=g["gpd"], radii=radii, blocks=blocks.tolist(),
                         levels=sorted(set(blocks[:, 0].tolist())),
                         written=int(written.sum()),
                         table_entries=int(len(g["tables"][1])), tables_sha256=th.hexdigest(),
                         sha256_written=hashlib.sha256(
                             np.ascontiguousarray(g["dump"][written], dtype="<f8").tobytes()).hexdigest())
        if written.all():
            out[name]["sha256"] = sha(g["dump"])
    with open(os.path.join(HERE, "dump_ref.json"), "w") as f:
        json.dump(out, f)


ADAPTIVE64 = dict(Dw=0.0013, rho=0.15, tend=110.0, L=6.4, dumpfreq=10.0, bpd=4, max_level=2,
                  seed_xyz=(20.3, 24.6, 22.1), peak=0.5, sigma=1.5)


def adaptive_phi_sha(blocks, phi):
    """SHA-256 of the block densities in (level, ix, iy, iz) order."""
    order = sorted(range(len(blocks)), key=lambda i: tuple(blocks[i]))
    h = hashlib.sha256()
    for i in order:
        h.update(np.ascontiguousarray(phi[i], dtype="<f8").tobytes())
    return h.hexdigest()


def adaptive_fixture():
    """The reference's adaptive run (ref_harness solve, -adaptive 1, the
    Glioma_HG_UQ::run loop with its final refinement) on the 64^3 anatomy:
    regrids every 10 days to 110 days, refinements and compressions both
    happen; step and regrid counts, final blocks and a hash of their
    densities, FP64 and the default FP32 build."""
    a = np.load(os.path.join(HERE, "anatomy64.npz"))
    pw, pg = a["p_w"].astype(np.float64), a["p_g"].astype(np.float64)
    an = S.Anatomy(n=64, p_w=pw, p_g=pg, psi=None)
    c = ADAPTIVE64
    phi0 = f32(S.gaussian_ic(an, *c["seed_xyz"], peak=c["peak"], sigma=c["sigma"]))
    out = {"params": c}
    for variant in ("f64", "f32"):
        r = refio.run_harness("solve", f"{variant}_l2", 64, c["bpd"], pw, pg, phi0, c["Dw"], c["rho"],
                              c["tend"], c["L"], adaptive=1, dumpfreq=c["dumpfreq"])
        blocks = [[b["level"], *b["index"]] for b in r["blocks"]]
        out[variant] = dict(steps=r["steps"], regrids=r["regrids"], blocks=sorted(blocks),
                            phi_sha256=adaptive_phi_sha(blocks, [b["phi"] for b in r["blocks"]]))
    with open(os.path.join(HERE, "adaptive64.json"), "w") as f:
        json.dump(out, f)


def patient_files(d, pat):
    """Write a synthetic patient the way the reference's `brain` reads it:
    <d>/Anatmoy/Patient01/P01_{GM,WM,CSF,T1,T2}.dat; returns the work folder
    <d>/run/work (the reference opens ../../Anatmoy/... from there)."""
    folder = os.path.join(d, "Anatmoy", "Patient01")
    os.makedirs(folder)
    for k in ("GM", "WM", "CSF", "T1", "T2"):
        matrix_io.write_d3d(os.path.join(folder, f"P01_{k}.dat"), pat[k].astype(np.float64))
    work = os.path.join(d, "run", "work")
    os.makedirs(work)
    np.array(pat["ic"], dtype="<f4").tofile(os.path.join(work, "HGG_TumorIC.bin"))
    with open(os.path.join(work, "HGG_InputParameters.txt"), "w") as f:
        f.write("\n".join(repr(float(x)) for x in pat["params"]) + "\n")
    return work


def synthetic_patient():
    """32^3 patient anatomy (float32-exact values): GM/WM from the seeded
    anatomy, a CSF pocket, T1/T2 lesion masks around the tumour centre."""
    an = S.make_anatomy(32, seed=5)
    n = 32
    z, y, x = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    r = np.sqrt((x - 20.0) ** 2 + (y - 14.0) ** 2 + (z - 16.0) ** 2)
    csf = np.where((r < 3.5) & an.brain, 0.6, 0.0)
    rt = np.sqrt((x - 15.0) ** 2 + (y - 17.0) ** 2 + (z - 15.0) ** 2)
    t1 = (rt < 1.5).astype(np.float64)
    t2 = (rt < 2.5).astype(np.float64)
    return dict(GM=f32(an.p_g), WM=f32(an.p_w), CSF=f32(csf), T1=t1, T2=t2,
                ic=[15.2 / 32, 17.1 / 32, 15.3 / 32], params=[0.0013, 0.2, 60.0])


def cli_fixture():
    """The reference's own `brain` (Glioma_HG_UQ.cpp built unmodified, FP32,
    4^3 blocks) and `likelihood` on a synthetic patient: hashes and values
    for gbg_brain / gbg_likelihood."""
    pat = synthetic_patient()
    out = {}
    with tempfile.TemporaryDirectory() as td:
        work = patient_files(td, pat)
        subprocess.run([os.path.join(refio.REF_DIR, "brain"), "-anatomy", "HGG_UQ", "-pID", "1",
                        "-adaptive", "0", "-dumpfreq", "1000", "-vtk", "0", "-verbose", "0",
                        "-nthreads", "1"], cwd=work, check=True, capture_output=True)
        u = matrix_io.read_d3d(os.path.join(work, "HGG_data.dat"))
        out["brain"] = dict(sha256=sha(u), sum=float(u.sum()), max=float(u.max()), n=u.shape[0])
        obs = cli_observations(u)
        for k, v in obs.items():
            if k == "Sphere":
                matrix_io.write_d2d(os.path.join(work, "Sphere.dat"), v)
            else:
                matrix_io.write_d3d(os.path.join(work, f"{k}_data.dat"), v)
        with open(os.path.join(work, "LikelihoodInput.txt"), "w") as f:
            f.write("\n".join(repr(x) for x in LIK_PARAMS) + "\n")
        p = subprocess.run([os.path.join(refio.REF_DIR, "likelihood")], cwd=work,
                           capture_output=True, text=True, check=True)
        out["likelihood"] = float(open(os.path.join(work, "Likelihood.txt")).read().split()[0])
        out["likelihood_stdout"] = p.stdout.strip().splitlines()[-3:]
        # the initial state alone: tend < 0 takes no step
        with open(os.path.join(work, "HGG_InputParameters.txt"), "w") as f:
            f.write("0.0013\n0.2\n-1\n")
        subprocess.run([os.path.join(refio.REF_DIR, "brain"), "-anatomy", "HGG_UQ", "-pID", "1",
                        "-adaptive", "0", "-dumpfreq", "1000", "-vtk", "0", "-verbose", "0",
                        "-nthreads", "1"], cwd=work, check=True, capture_output=True)
        u0 = matrix_io.read_d3d(os.path.join(work, "HGG_data.dat"))
        out["brain_ic"] = dict(sha256=sha(u0), sum=float(u0.sum()), max=float(u0.max()))
    np.savez_compressed(os.path.join(HERE, "patient32.npz"),
                        **{k: np.asarray(v, dtype=np.float32) for k, v in pat.items()
                           if k in ("GM", "WM", "CSF", "T1", "T2")},
                        ic=np.array(pat["ic"], dtype=np.float32), params=np.array(pat["params"]))
    with open(os.path.join(HERE, "patient32.json"), "w") as f:
        json.dump(out, f, indent=1)


def cli_adaptive_fixture():
    """The reference's `brain` built with _MAXLEVEL_ = 2 (its 4 blocks per
    dimension) run with -adaptive 1 -dumpfreq 10 on the synthetic patient:
    the hash of its HGG_data.dat, added to patient32.json."""
    pat = synthetic_patient()
    with tempfile.TemporaryDirectory() as td:
        work = patient_files(td, pat)
        subprocess.run([os.path.join(refio.REF_DIR, "brain_l2"), "-anatomy", "HGG_UQ", "-pID", "1",
                        "-adaptive", "1", "-dumpfreq", "10", "-vtk", "0", "-verbose", "0",
                        "-nthreads", "1"], cwd=work, check=True, capture_output=True)
        u = matrix_io.read_d3d(os.path.join(work, "HGG_data.dat"))
    path = os.path.join(HERE, "patient32.json")
    with open(path) as f:
        out = json.load(f)
    out["brain_adaptive"] = dict(sha256=sha(u), sum=float(u.sum()), max=float(u.max()), dumpfreq=10.0,
                                 max_level=2)
    with open(path, "w") as f:
        json.dump(out, f, indent=1)


PROPAGATION = [dict(n=64, S=12, seed=31), dict(n=32, S=3, seed=32), dict(n=32, S=1, seed=33)]


def propagation_fields(n, S, seed):
    """S seeded density-like fields [S, z, y, x] (float32): zero on a random
    30% of the cells, elsewhere a scaled, noisy copy of one base field in
    [0, 1]."""
    rng = np.random.default_rng(seed)
    base = rng.random((n, n, n))
    out = [np.where(base > 0.3, np.clip(base * rng.uniform(0.5, 1.5) + rng.normal(0, 0.05, (n, n, n)), 0, 1),
                    0.0).astype(np.float32) for _ in range(S)]
    return np.stack(out)


def propagation_fixture():
    """The reference's own `propagation` program (Glioma_HG_Propagation.cpp
    built unmodified, FP32) on seeded fields written as the S samples'
    HGG_data.dat: hashes of its PropagationMean_S.dat / PropagationVar_S.dat.
    The 32^3 cases use the tool built for 2 blocks per dimension."""
    pat = synthetic_patient()
    out = []
    for case in PROPAGATION:
        n, nS = case["n"], case["S"]
        fields = propagation_fields(n, nS, case["seed"])
        with tempfile.TemporaryDirectory() as td:
            work = patient_files(td, pat)
            folder = os.path.join(td, "Anatmoy", "Patient01", "Patient01_All_4K_Ti_step_3_mpp1")
            for s in range(nS):
                d = os.path.join(folder, f"tmpdir.0.0.0.{s}")
                os.makedirs(d)
                matrix_io.write_d3d(os.path.join(d, "HGG_data.dat"), fields[s].astype(np.float64))
            np.array([nS], dtype="<f4").tofile(os.path.join(work, "HGG_Nsamples.bin"))
            prog = "propagation" if n == 64 else "propagation_b2"
            subprocess.run([os.path.join(refio.REF_DIR, prog), "-anatomy", "HGG_Propagation", "-IC", "1",
                            "-pID", "1", "-vtk", "0", "-verbose", "0", "-nthreads", "1"],
                           cwd=work, check=True, capture_output=True)
            mean = matrix_io.read_d3d(os.path.join(work, f"PropagationMean_{nS}.dat"))
            var = matrix_io.read_d3d(os.path.join(work, f"PropagationVar_{nS}.dat"))
        assert mean.shape == (n, n, n)
        out.append(dict(case, mean_sha256=sha(mean), var_sha256=sha(var), mean_sum=float(mean.sum()),
                        var_sum=float(var.sum()), mean_center=float(mean[n // 2, n // 3, n // 4]),
                        var_center=float(var[n // 2, n // 3, n // 4])))
    with open(os.path.join(HERE, "propagation.json"), "w") as f:
        json.dump(out, f, indent=1)


SYNTHETIC = [dict(n=64, centre=(30.3, 35.1, 28.7), radius=9.0), dict(n=32, centre=(14.6, 17.2, 15.9), radius=6.5)]


def synthetic_tumour(n, centre, radius):
    """A tumour-like density on n^3 made with correctly rounded operations
    only (+, -, *, /, sqrt and integer arithmetic), so any platform makes the
    same bits: a linear fall-off from 1.05 at the centre to 0 at twice the
    radius, plus a +-0.02 integer-hash texture, clipped to [0, 1], as float
    values."""
    z, y, x = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    r = np.sqrt((x - centre[0]) ** 2 + (y - centre[1]) ** 2 + (z - centre[2]) ** 2)
    h = ((7 * x + 13 * y + 29 * z + 3 * x * y + 5 * y * z) % 1009).astype(np.float64) / 1009.0
    u = np.clip(1.05 - r / (2.0 * radius) * 1.05 + 0.04 * (h - 0.5), 0.0, 1.0)
    return u.astype(np.float32).astype(np.float64)


def synthetic_fixture():
    """The reference's own synthetic-data program (Glioma_ProcessSyntheticData
    built unmodified, FP32, through oracle/synthetic_main.cpp, which also
    writes the grid's block loop order) on seeded tumours: hashes of its
    PET/T1/T2_data.dat, its HGG_TumorIC.bin centre of mass and the block
    order. The 32^3 case uses the program built for 2 blocks per dimension."""
    out = []
    for case in SYNTHETIC:
        n = case["n"]
        u = synthetic_tumour(n, case["centre"], case["radius"])
        with tempfile.TemporaryDirectory() as td:
            matrix_io.write_d3d(os.path.join(td, "HGG_data.dat"), u)
            prog = "synthetic" if n == 64 else "synthetic_b2"
            subprocess.run([os.path.join(refio.REF_DIR, prog), "-anatomy", "syntheticData", "-adaptive", "0",
                            "-vtk", "0", "-verbose", "0", "-nthreads", "1"], cwd=td, check=True, capture_output=True)
            res = {k: matrix_io.read_d3d(os.path.join(td, f"{k}_data.dat")) for k in ("PET", "T1", "T2")}
            com = np.fromfile(os.path.join(td, "HGG_TumorIC.bin"), dtype="<f4")[:3]
            order = np.loadtxt(os.path.join(td, "block_order.txt"), dtype=int).reshape(-1, 4)
        out.append(dict(case, tumour_cells=int((u.astype(np.float32) >= np.float32(0.3)).sum()),
                        block_order=order.tolist(), centre_of_mass=[float(c) for c in com],
                        **{f"{k.lower()}_sha256": sha(v) for k, v in res.items()},
                        pet_sum=float(res["PET"].sum())))
    with open(os.path.join(HERE, "synthetic.json"), "w") as f:
        json.dump(out, f)


def cli_observations(u):
    """Observations of a model field, deterministic from a seed (numpy only)."""
    rng = np.random.default_rng(21)
    t1 = (u > 0.7).astype(np.float64)
    t2 = (u > 0.25).astype(np.float64)
    pet = np.where(u > 0, np.maximum(0.0, u + rng.normal(0, 0.05, u.shape)), 0.0)
    zz, yy, xx = np.nonzero(u > 1e-6)
    pts = np.stack([xx, yy, zz], axis=0).astype(np.float64)  # D2D: row j = coordinate j
    return dict(PET=pet, T1=t1, T2=t2, Sphere=pts)


if __name__ == "__main__":
    if len(sys.argv) > 1 and sys.argv[1] == "mala":
        mala_fixture()
        sys.exit(0)
    if len(sys.argv) > 1 and sys.argv[1] == "dump":
        dump_fixtures()
        sys.exit(0)
    if len(sys.argv) > 1 and sys.argv[1] == "propagation":
        propagation_fixture()
        sys.exit(0)
    if len(sys.argv) > 1 and sys.argv[1] == "synthetic":
        synthetic_fixture()
        sys.exit(0)
    if len(sys.argv) > 1 and sys.argv[1] == "adaptive":
        adaptive_fixture()
        cli_adaptive_fixture()
        sys.exit(0)
    rd_fixtures()
    mala_fixture()
    lik_fixture()
    amr_fixtures()
    dump_fixtures()
    adaptive_fixture()
    cli_fixture()
    cli_adaptive_fixture()
    propagation_fixture()
    synthetic_fixture()
    for f in sorted(os.listdir(HERE)):
        print(f, os.path.getsize(os.path.join(HERE, f)))
