"""CPU oracle for the multiresolution block grid -- TEST INFRASTRUCTURE ONLY.

NumPy restatement of what GliomaUQ does on MRAG's adaptive grid of 16^3
blocks, vectorised over blocks and cells with every operation in the
reference's Real type (IEEE single or double, one rounding per operation):

  * ghost values: BlockLab::load (source/MRAGcore/MRAGBlockLab.h:254-295),
    ghost = sum_k value_k * w_k from 0 in table order;
  * the step: Glioma_ReactionDiffusionOperator<3> Case2 + UpdateTumor<3>
    (source/Glioma/Glioma_ReactionDiffusionOperator.h:148-218, :254-261) on
    each block's 18^3 lab with h = 1/(2^level * 16);
  * the FWT detail maximum: BlockFWT::_filter/_fwt + FWTReport
    (source/MRAGcore/MRAGBlockFWT.h:184-190, 219-298), Interp2ndOrder filters.

Pinned against the reference's own outputs in tests/golden/amr64_*.npz.
"""
from __future__ import annotations

import numpy as np

BS = 16
NG = 1736


def region_starts():
    out, start = [], 0
    for c in range(27):
        d = (c % 3 - 1, (c // 3) % 3 - 1, (c // 9) % 3 - 1)
        size = int(np.prod([BS if x == 0 else 1 for x in d]))
        out.append(start if c != 13 else -1)
        if c != 13:
            start += size
    return out


def _lab_slots():
    """(18,18,18) map from lab cell (z+1, y+1, x+1) to ghost slot (-1 inside)."""
    rs = region_starts()
    m = np.full((18, 18, 18), -1, dtype=np.int64)
    for z in range(-1, 17):
        for y in range(-1, 17):
            for x in range(-1, 17):
                if 0 <= x < BS and 0 <= y < BS and 0 <= z < BS:
                    continue
                d = [(-1 if v < 0 else (1 if v >= BS else 0)) for v in (x, y, z)]
                code = (d[0] + 1) + 3 * (d[1] + 1) + 9 * (d[2] + 1)
                n0 = BS if d[0] == 0 else 1
                n1 = BS if d[1] == 0 else 1
                lx = x if d[0] == 0 else 0
                ly = y if d[1] == 0 else 0
                lz = z if d[2] == 0 else 0
                m[z + 1, y + 1, x + 1] = rs[code] + lx + n0 * (ly + n1 * lz)
    return m


LAB_SLOTS = _lab_slots()


def ghost_values(field, start, src_block, src_cell, w, real):
    """field: (nb, 4096) in `real`; returns (nb*1736,) ghost values."""
    f = np.asarray(field, dtype=real).reshape(-1)
    start = np.asarray(start, dtype=np.int64)
    counts = np.diff(start)
    acc = np.zeros(counts.size, dtype=real)
    src = np.asarray(src_block, dtype=np.int64) * 4096 + np.asarray(src_cell, dtype=np.int64)
    ww = np.asarray(w, dtype=real)
    for k in range(int(counts.max()) if counts.size else 0):
        sel = np.nonzero(counts > k)[0]
        e = start[sel] + k
        acc[sel] = acc[sel] + f[src[e]] * ww[e]
    return acc


def labs(field, ghosts, real):
    """(nb, 18, 18, 18) labs, index [b, z+1, y+1, x+1]."""
    f = np.asarray(field, dtype=real).reshape(-1, BS, BS, BS)
    g = np.asarray(ghosts, dtype=real).reshape(f.shape[0], NG)
    out = np.empty((f.shape[0], 18, 18, 18), dtype=real)
    inside = LAB_SLOTS < 0
    out[:, 1:17, 1:17, 1:17] = f
    idx = np.nonzero(~inside)
    out[:, idx[0], idx[1], idx[2]] = g[:, LAB_SLOTS[idx]]
    return out


def step(levels, pw, pg, phi, ghost_tables, Dw, Dg, rho, dt, real):
    """One step on every block; returns the new phi (nb, 16, 16, 16) in `real`."""
    st, sb, sc, w = ghost_tables
    real = np.dtype(real).type
    Lw = labs(pw, ghost_values(pw, st, sb, sc, w, real), real)
    Lg = labs(pg, ghost_values(pg, st, sb, sc, w, real), real)
    Lp = labs(phi, ghost_values(phi, st, sb, sc, w, real), real)
    Dw, Dg, rho = real(Dw), real(Dg), real(rho)
    c = (slice(None), slice(1, 17), slice(1, 17), slice(1, 17))
    sh = {0: (0, 0, -1), 1: (0, 0, 1), 2: (0, -1, 0), 3: (0, 1, 0), 4: (-1, 0, 0), 5: (1, 0, 0)}

    def at(L, f):
        dz, dy, dx = sh[f]
        return L[:, 1 + dz:17 + dz, 1 + dy:17 + dy, 1 + dx:17 + dx]

    with np.errstate(all="ignore"):
        brain0 = Lw[c] + Lg[c]
        inv0 = 1.0 / ((Lw[c] * Dw + Lg[c] * Dg) / brain0).astype(np.float64)
        tissue = brain0 + Lp[c]
        df = []
        for f in range(6):
            bn = at(Lw, f) + at(Lg, f)
            kn = (at(Lw, f) * Dw + at(Lg, f) * Dg) / bn
            d = 2.0 * (1.0 / (inv0 + 1.0 / kn.astype(np.float64)))
            df.append(np.where(tissue > 0, d, 0.0))
        pn = [at(Lp, f).astype(np.float64) for f in range(6)]
        pairs = [(0, 1, 0), (1, 0, 1), (2, 3, 2), (3, 2, 3), (4, 5, 4), (5, 4, 5)]
        for zf, other, nb in pairs:
            df[other] = np.where((df[zf] == 0) & (pn[nb] > 0), df[other] * 2.0, df[other])
        h = np.array([real(1) / real((1 << int(l)) * BS) for l in levels], dtype=np.float64)
        ih2 = (1.0 / (h * h))[:, None, None, None]
        p0 = Lp[c]
        fin = ih2 * (df[0] * pn[0] + df[1] * pn[1] + df[2] * pn[2] + df[3] * pn[3] + df[4] * pn[4]
                     + df[5] * pn[5])
        fout = -((df[0] + df[1] + df[2] + df[3] + df[4] + df[5]) * p0.astype(np.float64) * ih2)
        react = (rho * p0).astype(np.float64) * (1.0 - p0.astype(np.float64))
        dphidt = (fout + fin + react).astype(real)
        v = (p0.astype(np.float64) + dt * dphidt.astype(np.float64)).astype(real)
    v = np.where(real(0) < v, v, real(0))
    v = np.where(v < real(1), v, real(1))
    return v.astype(real)


def fwt_detail(phi, ghost_tables, real):
    """Per-block largest detail magnitude of the one-level interpolating
    wavelet transform of phi (FWTReport::getOverAll_DetailMaxMag)."""
    st, sb, sc, w = ghost_tables
    real = np.dtype(real).type
    L = labs(phi, ghost_values(phi, st, sb, sc, w, real), real)
    ga = {-2: real(-0.5), -1: real(1.0), 0: real(-0.5)}
    d = np.arange(8)
    out = np.zeros(L.shape[0], dtype=np.float64)
    for sbnd in range(1, 8):
        wx, wy, wz = sbnd & 1, (sbnd >> 1) & 1, (sbnd >> 2) & 1
        rx = [-2, -1, 0] if wx else [0]
        ry = [-2, -1, 0] if wy else [0]
        rz = [-2, -1, 0] if wz else [0]
        res = np.zeros((L.shape[0], 8, 8, 8), dtype=real)
        for iz in rz:
            wZ = ga[iz] if wz else real(1)
            for iy in ry:
                wY = ga[iy] if wy else real(1)
                wZwY = real(wZ * wY)
                for ix in rx:
                    wX = ga[ix] if wx else real(1)
                    zz, yy, xx = 2 * d - iz + 1, 2 * d - iy + 1, 2 * d - ix + 1
                    v = L[:, zz][:, :, yy][:, :, :, xx]
                    res = res + v * real(wZwY * wX)
        out = np.maximum(out, np.abs(res.astype(np.float64)).reshape(L.shape[0], -1).max(axis=1))
    return out


def remap_plan(old_blocks, new_blocks):
    """kind/src arrays of gbg_amr_remap that turn the grid `old_blocks` into
    `new_blocks` ((n, 4) arrays of level, ix, iy, iz), found by position."""
    pos = {tuple(b): i for i, b in enumerate(np.asarray(old_blocks).tolist())}
    kind = np.zeros(len(new_blocks), dtype=np.int32)
    src = np.zeros((len(new_blocks), 8), dtype=np.int32)
    for i, (l, x, y, z) in enumerate(np.asarray(new_blocks).tolist()):
        if (l, x, y, z) in pos:
            kind[i], src[i, 0] = 0, pos[(l, x, y, z)]
        elif (l - 1, x // 2, y // 2, z // 2) in pos:
            kind[i] = 1
            src[i, 0] = pos[(l - 1, x // 2, y // 2, z // 2)]
            src[i, 1] = (x % 2) + 2 * (y % 2) + 4 * (z % 2)
        else:
            kids = [(l + 1, 2 * x + (c & 1), 2 * y + ((c >> 1) & 1), 2 * z + ((c >> 2) & 1))
                    for c in range(8)]
            if not all(k in pos for k in kids):
                raise ValueError(f"block {(l, x, y, z)} is not a copy, split or collapse")
            kind[i] = 2
            src[i] = [pos[k] for k in kids]
    return kind, src


def remap(field, ghosts, kind, src, real):
    """BlockSplitter / BlockCollapser data movement of one field
    (source/MRAGcore/MRAGBlockSplitter.h:24-100, MRAGBlockCollapser.h:19-61)."""
    real = np.dtype(real).type
    f = np.asarray(field, dtype=real).reshape(-1, BS, BS, BS)
    L = labs(f.reshape(-1, 4096), ghosts, real)
    out = np.empty((len(kind), BS, BS, BS), dtype=real)
    fine = np.arange(2 * BS)
    for i, k in enumerate(kind):
        if k == 0:
            out[i] = f[src[i][0]]
        elif k == 1:
            p, ch = src[i][0], src[i][1]
            off = [(ch & 1) * BS, ((ch >> 1) & 1) * BS, ((ch >> 2) & 1) * BS]
            d = [fine[o:o + BS] for o in off]  # fine indices per axis
            acc = np.zeros((BS, BS, BS), dtype=real)
            # per axis: first parent point and its weight, second (odd d only)
            lo = [dd // 2 for dd in d]
            odd = [dd % 2 == 1 for dd in d]
            for iz in (0, 1):
                for iy in (0, 1):
                    for ix in (0, 1):
                        use = (odd[2] | (iz == 0))[:, None, None] & (odd[1] | (iy == 0))[None, :, None] \
                            & (odd[0] | (ix == 0))[None, None, :]
                        wz = np.where(odd[2], 0.5, 1.0)
                        wy = np.where(odd[1], 0.5, 1.0)
                        wx = np.where(odd[0], 0.5, 1.0)
                        w = ((wz[:, None, None] * wy[None, :, None]) * wx[None, None, :]).astype(real)
                        zz = (lo[2] + iz)[:, None, None] + 1
                        yy = (lo[1] + iy)[None, :, None] + 1
                        xx = (lo[0] + ix)[None, None, :] + 1
                        v = L[p][np.minimum(zz, 17), np.minimum(yy, 17), np.minimum(xx, 17)]
                        acc = np.where(use, acc + v * w, acc)
            out[i] = acc
        else:
            for c in range(8):
                cz, cy, cx = (c >> 2) & 1, (c >> 1) & 1, c & 1
                out[i, cz * 8:(cz + 1) * 8, cy * 8:(cy + 1) * 8, cx * 8:(cx + 1) * 8] = \
                    real(0) + f[src[i][c], ::2, ::2, ::2] * real(1.0)
    return out


def dump_uniform(blocks, phi, gpd, reference_rules=True):
    """Glioma_HG_UQ::_dumpUQoutput (source/Glioma/Glioma_HG_UQ.cpp:309-372):
    every block cell replicated r^3 times on the gpd^3 grid, r = 1 for h = hf,
    2 for h = 2 hf, 3 for h = 3 hf and 4 otherwise (reference_rules), or
    exactly h / hf; unwritten cells are 0."""
    out = np.zeros((gpd, gpd, gpd))
    f = np.asarray(phi, dtype=np.float64).reshape(-1, BS, BS, BS)
    for i, (l, bx, by, bz) in enumerate(np.asarray(blocks).tolist()):
        cells = BS << l
        if cells >= gpd:
            ratio = cells // gpd
            sub = f[i][::ratio, ::ratio, ::ratio] if ratio > 1 else f[i]
            # only the cells whose global index is a multiple of ratio
            g0 = np.array([bz, by, bx]) * BS
            first = (-g0) % ratio
            sub = f[i][first[0]::ratio, first[1]::ratio, first[2]::ratio]
            m = (g0 + first) // ratio
            out[m[0]:m[0] + sub.shape[0], m[1]:m[1] + sub.shape[1], m[2]:m[2] + sub.shape[2]] = sub
            continue
        ratio = gpd // cells
        r = ratio if not reference_rules else (ratio if ratio in (1, 2, 3) else 4)
        # cell (z, y, x) of the block writes the r^3 cells starting at
        # ((b * BS + z) * ratio, ...); viewed as (BS, ratio)^3 the block's
        # region takes the first r of every ratio
        span = BS * ratio
        reg = out[bz * span:(bz + 1) * span, by * span:(by + 1) * span, bx * span:(bx + 1) * span]
        reg = reg.reshape(BS, ratio, BS, ratio, BS, ratio)
        reg[:, :r, :, :r, :, :r] = f[i][:, None, :, None, :, None]
    return out
