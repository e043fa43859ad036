"""Test infrastructure only: file formats of oracle/ref_harness.cpp and a
runner for the reference binaries compiled into oracle/_ref/."""
from __future__ import annotations

import os
import struct
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
# The reference's source tree (GliomaUQ's source/ folder), read only by the
# recipes that compile it in place and by the tests that need it; override
# with GLIOMAUQ_REF. oracle/Makefile takes the same variable.
REF_SOURCE = os.environ.get("GLIOMAUQ_REF", "/root/reference/source")


def write_input(path, n, bpd, pw, pg, phi, Dw_file, rho, tend, L, adaptive=0, nsteps=-1,
                dumpfreq=1e30):
    with open(path, "wb") as f:
        f.write(b"GBGREF01")
        f.write(struct.pack("<4i", n, bpd, adaptive, nsteps))
        f.write(struct.pack("<5d", Dw_file, rho, tend, L, dumpfreq))
        for a in (pw, pg, phi):
            np.ascontiguousarray(a, dtype="<f8").tofile(f)


def read_solve_output(path):
    raw = open(path, "rb").read()
    assert raw[:8] == b"GBGOUT01"
    n, real_bytes, steps, regrids = struct.unpack_from("<4i", raw, 8)
    dt, dw, dg, rho = struct.unpack_from("<4d", raw, 24)
    off = 56
    N = n ** 3
    u = np.frombuffer(raw, "<f8", N, off).reshape(n, n, n).copy()
    off += 8 * N
    (nb,) = struct.unpack_from("<i", raw, off)
    off += 4
    blocks = []
    for _ in range(nb):
        bid, lvl, ix, iy, iz = struct.unpack_from("<5i", raw, off)
        off += 20
        d = np.frombuffer(raw, "<f8", 3 * 4096, off).reshape(3, 16, 16, 16).copy()
        off += 8 * 3 * 4096
        blocks.append(dict(id=bid, level=lvl, index=(ix, iy, iz), phi=d[0], p_w=d[1], p_g=d[2]))
    return dict(n=n, real_bytes=real_bytes, steps=steps, regrids=regrids, dt=dt, Dw=dw, Dg=dg,
                rho=rho, phi=u, blocks=blocks)


def read_mala_output(path):
    """Output of `ref_harness mala`: phi, sRho, sD on the uniform grid."""
    raw = open(path, "rb").read()
    assert raw[:8] == b"GBGMAL01"
    n, real_bytes, steps, _ = struct.unpack_from("<4i", raw, 8)
    dt, dw, dg, rho = struct.unpack_from("<4d", raw, 24)
    off = 56
    N = n ** 3
    f = [np.frombuffer(raw, "<f8", N, off + 8 * N * k).reshape(n, n, n).copy() for k in range(3)]
    return dict(n=n, real_bytes=real_bytes, steps=steps, dt=dt, Dw=dw, Dg=dg, rho=rho,
                phi=f[0], sRho=f[1], sD=f[2])


def read_ghosts(path):
    raw = open(path, "rb").read()
    assert raw[:8] == b"GBGGHO01"
    off = 8
    (nb,) = struct.unpack_from("<i", raw, off)
    off += 4
    out = []
    for _ in range(nb):
        bid, lvl, ix, iy, iz, ng = struct.unpack_from("<6i", raw, off)
        off += 24
        regions = np.frombuffer(raw, "<i4", 54, off).reshape(27, 2).copy()
        off += 4 * 54
        ghosts = []
        for _g in range(ng):
            (cnt,) = struct.unpack_from("<i", raw, off)
            off += 4
            items = []
            for _k in range(cnt):
                sb, si = struct.unpack_from("<2i", raw, off)
                w = struct.unpack_from("<3d", raw, off + 8)
                off += 32
                items.append((sb, si, w[0], w[1], w[2]))
            ghosts.append(items)
        out.append(dict(id=bid, level=lvl, index=(ix, iy, iz), regions=regions, ghosts=ghosts))
    return out


def read_fwt(path):
    raw = open(path, "rb").read()
    assert raw[:8] == b"GBGFWT01"
    (nb,) = struct.unpack_from("<i", raw, 8)
    off = 12
    out = []
    for _ in range(nb):
        bid, lvl, ix, iy, iz = struct.unpack_from("<5i", raw, off)
        (d,) = struct.unpack_from("<d", raw, off + 20)
        off += 28
        out.append(dict(id=bid, level=lvl, index=(ix, iy, iz), detail=d))
    return out


def run_harness(cmd, variant, n, bpd, pw, pg, phi, Dw_file, rho, tend, L, adaptive=0,
                nsteps=-1, dumpfreq=1e30, timeout=3600):
    exe = os.path.join(REF_DIR, f"ref_harness_{variant}")
    if not os.path.exists(exe):
        raise FileNotFoundError(exe)
    with tempfile.TemporaryDirectory() as td:
        inp = os.path.join(td, "in.bin")
        outp = os.path.join(td, "out.bin")
        write_input(inp, n, bpd, pw, pg, phi, Dw_file, rho, tend, L, adaptive, nsteps, dumpfreq)
        subprocess.run([exe, cmd, inp, outp], check=True, timeout=timeout,
                       stdout=subprocess.DEVNULL, stderr=subprocess.PIPE)
        if cmd == "solve":
            return read_solve_output(outp)
        if cmd == "mala":
            return read_mala_output(outp)
        if cmd == "ghosts":
            return read_ghosts(outp)
        if cmd == "fwt":
            return read_fwt(outp)
    raise ValueError(cmd)


def _read_blocks(raw, off):
    (nb,) = struct.unpack_from("<i", raw, off)
    off += 4
    blocks = []
    for _ in range(nb):
        bid, lvl, ix, iy, iz = struct.unpack_from("<5i", raw, off)
        off += 20
        d = np.frombuffer(raw, "<f8", 3 * 4096, off).reshape(3, 16, 16, 16).copy()
        off += 8 * 3 * 4096
        blocks.append(dict(id=bid, level=lvl, index=(ix, iy, iz), phi=d[0], p_w=d[1], p_g=d[2]))
    return blocks, off


def _read_ghost_tables(raw, off):
    """writeGhostTables output: per block its blockID, 27 region headers and
    per ghost the (source blockID, source cell, weight product) entries."""
    (nb,) = struct.unpack_from("<i", raw, off)
    off += 4
    rec = np.dtype([("b", "<i4"), ("c", "<i4"), ("w", "<f8")])
    ghosts = []
    for _ in range(nb):
        bid, ng = struct.unpack_from("<2i", raw, off)
        off += 8
        regions = np.frombuffer(raw, "<i4", 54, off).reshape(27, 2).copy()
        off += 4 * 54
        counts = np.empty(ng, dtype=np.int32)
        parts = []
        for g in range(ng):
            (cnt,) = struct.unpack_from("<i", raw, off)
            off += 4
            counts[g] = cnt
            if cnt:
                parts.append(np.frombuffer(raw, rec, cnt, off))
                off += 16 * cnt
        e = np.concatenate(parts) if parts else np.empty(0, dtype=rec)
        ghosts.append(dict(id=bid, regions=regions, counts=counts,
                           src_block=e["b"].astype(np.int32), src_cell=e["c"].astype(np.int32),
                           w=e["w"].astype(np.float64)))
    return ghosts, off


def flatten_tables(ghosts, ids):
    """The tables as gbg_amr_set_ghosts takes them, blocks in the order of
    `ids` (source blockIDs mapped to positions in that order)."""
    slot = {int(b): i for i, b in enumerate(ids)}
    by_id = {g["id"]: g for g in ghosts}
    counts = np.concatenate([by_id[int(b)]["counts"] for b in ids])
    start = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
    lut = np.vectorize(lambda x: slot[int(x)], otypes=[np.int32])
    sb = np.concatenate([lut(by_id[int(b)]["src_block"]) if by_id[int(b)]["src_block"].size
                         else np.empty(0, np.int32) for b in ids]).astype(np.int32)
    sc = np.concatenate([by_id[int(b)]["src_cell"] for b in ids]).astype(np.int32)
    w = np.concatenate([by_id[int(b)]["w"] for b in ids])
    return start, sb, sc, w


def read_state(path):
    """Output of `ref_harness state`: S0 blocks + ghost tables + FWT maxima,
    S1 blocks (after k more steps), S2 blocks (after one more regrid)."""
    raw = open(path, "rb").read()
    assert raw[:8] == b"GBGSTA01"
    n, real_bytes, steps, regrids = struct.unpack_from("<4i", raw, 8)
    dt, dw, dg, rho = struct.unpack_from("<4d", raw, 24)
    off = 56
    s0, off = _read_blocks(raw, off)
    (nb,) = struct.unpack_from("<i", raw, off)
    off += 4
    ghosts = []
    for _ in range(nb):
        bid, ng = struct.unpack_from("<2i", raw, off)
        off += 8
        regions = np.frombuffer(raw, "<i4", 54, off).reshape(27, 2).copy()
        off += 4 * 54
        counts = np.empty(ng, dtype=np.int32)
        src_b, src_c, w = [], [], []
        for g in range(ng):
            (cnt,) = struct.unpack_from("<i", raw, off)
            off += 4
            counts[g] = cnt
            for _k in range(cnt):
                sb, sc = struct.unpack_from("<2i", raw, off)
                (ww,) = struct.unpack_from("<d", raw, off + 8)
                off += 16
                src_b.append(sb)
                src_c.append(sc)
                w.append(ww)
        ghosts.append(dict(id=bid, regions=regions, counts=counts,
                           src_block=np.array(src_b, dtype=np.int32),
                           src_cell=np.array(src_c, dtype=np.int32), w=np.array(w)))
    (nb2,) = struct.unpack_from("<i", raw, off)
    off += 4
    fwt = np.frombuffer(raw, "<f8", nb2, off).copy()
    off += 8 * nb2
    s1, off = _read_blocks(raw, off)
    s2, off = _read_blocks(raw, off)
    return dict(n=n, real_bytes=real_bytes, steps=steps, regrids=regrids, dt=dt, Dw=dw, Dg=dg,
                rho=rho, s0=s0, ghosts=ghosts, fwt=fwt, s1=s1, s2=s2)


def run_state(variant, n, bpd, pw, pg, phi, Dw_file, rho, tend, L, dumpfreq, extra=10,
              timeout=3600):
    exe = os.path.join(REF_DIR, f"ref_harness_{variant}")
    with tempfile.TemporaryDirectory() as td:
        inp = os.path.join(td, "in.bin")
        outp = os.path.join(td, "out.bin")
        write_input(inp, n, bpd, pw, pg, phi, Dw_file, rho, tend, L, 1, -1, dumpfreq)
        subprocess.run([exe, "state", inp, outp, str(extra)], check=True, timeout=timeout,
                       stdout=subprocess.DEVNULL, stderr=subprocess.PIPE)
        return read_state(outp)


def run_dump(exe_name, n, bpd, pw, pg, phi, Dw_file, rho, tend, L, adaptive=1, nsteps=-1,
             dumpfreq=1e30, regrid=0, timeout=3600):
    """`ref_dump_* dump`: the time loop as `state` runs it (optionally one
    more regrid), the blocks of the resulting grid, and the reference's own
    Glioma_HG_UQ::_dumpUQoutput of that grid (HGG_data.dat, read back as a
    (gpd, gpd, gpd) array indexed [z, y, x])."""
    exe = os.path.join(REF_DIR, exe_name)
    with tempfile.TemporaryDirectory() as td:
        inp = os.path.join(td, "in.bin")
        outp = os.path.join(td, "out.bin")
        write_input(inp, n, bpd, pw, pg, phi, Dw_file, rho, tend, L, adaptive, nsteps, dumpfreq)
        subprocess.run([exe, "dump", inp, outp, str(int(regrid))], check=True, timeout=timeout,
                       cwd=td, stdout=subprocess.DEVNULL, stderr=subprocess.PIPE)
        raw = open(outp, "rb").read()
        assert raw[:8] == b"GBGDMP01"
        n_, real_bytes, steps, regrids = struct.unpack_from("<4i", raw, 8)
        (gpd,) = struct.unpack_from("<i", raw, 24)
        blocks, _ = _read_blocks(raw, 28)
        d = open(os.path.join(td, "HGG_data.dat"), "rb").read()
    # Matrix::D3D (Glioma/Matrix.h): ints {1234, 3, nx, ny, nz, type 0 = double},
    # then the values, x fastest
    magic, dim, sx, sy, sz, tid = struct.unpack_from("<6i", d, 0)
    assert magic == 1234 and dim == 3 and tid == 0, (magic, dim, tid)
    dump = np.frombuffer(d, "<f8", sx * sy * sz, 24).reshape(sz, sy, sx).copy()
    return dict(steps=steps, regrids=regrids, gpd=gpd, blocks=blocks, dump=dump)


def run_dumpgrid(exe_name, radii, timeout=3600):
    """`ref_dump_* dumpgrid`: the blocks (level, ix, iy, iz) of the forced
    multi-level grid and the reference's _dumpUQoutput of it (cells set by
    dumpgrid_phi)."""
    exe = os.path.join(REF_DIR, exe_name)
    with tempfile.TemporaryDirectory() as td:
        outp = os.path.join(td, "out.bin")
        subprocess.run([exe, "dumpgrid", outp, *[repr(float(r)) for r in radii]], cwd=td,
                       check=True, timeout=timeout, stdout=subprocess.DEVNULL,
                       stderr=subprocess.PIPE)
        raw = open(outp, "rb").read()
        assert raw[:8] == b"GBGDMP03"
        gpd, nb = struct.unpack_from("<2i", raw, 8)
        hdr = np.frombuffer(raw, "<i4", 5 * nb, 16).reshape(nb, 5).copy()
        ids, blocks = hdr[:, 0], hdr[:, 1:]
        ghosts, _ = _read_ghost_tables(raw, 16 + 20 * nb)
        d = open(os.path.join(td, "HGG_data.dat"), "rb").read()
    magic, dim, sx, sy, sz, tid = struct.unpack_from("<6i", d, 0)
    assert magic == 1234 and dim == 3 and tid == 0, (magic, dim, tid)
    dump = np.frombuffer(d, "<f8", sx * sy * sz, 24).reshape(sz, sy, sx).copy()
    return dict(gpd=gpd, blocks=blocks, dump=dump, tables=flatten_tables(ghosts, ids))


def dumpgrid_phi(blocks):
    """The cell values `dumpgrid` sets: ((7 gx + 13 gy + 29 gz + 101 level) mod
    1009) / 1009 with (gx, gy, gz) the cell's index on its level; (nb, 16, 16,
    16) indexed [block, z, y, x]."""
    b = np.asarray(blocks, dtype=np.int64)
    z, y, x = np.meshgrid(np.arange(16), np.arange(16), np.arange(16), indexing="ij")
    out = np.empty((b.shape[0], 16, 16, 16))
    for i, (lv, ix, iy, iz) in enumerate(b.tolist()):
        out[i] = ((7 * (ix * 16 + x) + 13 * (iy * 16 + y) + 29 * (iz * 16 + z) + 101 * lv)
                  % 1009) / 1009.0
    return out
