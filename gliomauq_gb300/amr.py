"""Host-side helpers for the multiresolution block grid (gbg_amr_*).

MRAG's ghost instruction tables for grids with resolution jumps are compiled
by MRAG itself (MRAG_BBInfoCreator, source/MRAGcore/MRAG_BBInfoCreator.inl)
and handed to the library at the drop-in boundary. For a grid whose blocks
all sit at one level the tables reduce to periodic copies, which this module
builds directly, in the ghost order of BlockLab::load
(source/MRAGcore/MRAGBlockLab.h:256-295): the 26 neighbour regions by code
(x fastest, the centre skipped), each region z-y-x, for the stencil [-1, 2).
"""
from __future__ import annotations

import numpy as np

BS = 16
NG = 1736  # ghost cells per block for the stencil [-1, 2)


def ghost_lab_coords() -> np.ndarray:
    """(1736, 3) lab coordinates (x, y, z), each in [-1, 16], in ghost order."""
    out = []
    for code in range(27):
        if code == 13:
            continue
        d = (code % 3 - 1, (code // 3) % 3 - 1, (code // 9) % 3 - 1)
        rng = [range(BS) if v == 0 else [(-1 if v < 0 else BS)] for v in d]
        for z in rng[2]:
            for y in rng[1]:
                for x in rng[0]:
                    out.append((x, y, z))
    a = np.array(out, dtype=np.int64)
    assert a.shape == (NG, 3)
    return a


def uniform_blocks(level: int) -> np.ndarray:
    """(nb, 4) blocks (level, ix, iy, iz) of a one-level grid, ix fastest."""
    m = 1 << level
    iz, iy, ix = np.meshgrid(np.arange(m), np.arange(m), np.arange(m), indexing="ij")
    nb = m ** 3
    return np.stack([np.full(nb, level), ix.ravel(), iy.ravel(), iz.ravel()], axis=1).astype(np.int32)


def to_block_major(field: np.ndarray, level: int) -> np.ndarray:
    """[z, y, x] uniform field (n = 16 * 2^level) -> (nb * 4096,) block-major,
    blocks in uniform_blocks order, x fastest inside a block."""
    m = 1 << level
    f = np.asarray(field).reshape(m, BS, m, BS, m, BS)  # bz, z, by, y, bx, x
    return np.ascontiguousarray(f.transpose(0, 2, 4, 1, 3, 5)).reshape(-1)


def from_block_major(blocks_field: np.ndarray, level: int) -> np.ndarray:
    m = 1 << level
    f = np.asarray(blocks_field).reshape(m, m, m, BS, BS, BS)  # bz, by, bx, z, y, x
    return np.ascontiguousarray(f.transpose(0, 3, 1, 4, 2, 5)).reshape(m * BS, m * BS, m * BS)


def same_level_ghosts(blocks: np.ndarray):
    """Ghost tables (start, src_block, src_cell, w) of a periodic grid whose
    blocks all have one level and tile the unit cube: every ghost is a copy
    (one term, weight 1) of the cell of the neighbouring block at the same
    place."""
    b = np.asarray(blocks, dtype=np.int64)
    level = int(b[0, 0])
    if np.any(b[:, 0] != level):
        raise ValueError("same_level_ghosts needs every block at one level")
    m = 1 << level
    if b.shape[0] != m ** 3:
        raise ValueError("the blocks must tile the unit cube")
    ids = np.full((m, m, m), -1, dtype=np.int64)  # [iz, iy, ix] -> block id
    ids[b[:, 3], b[:, 2], b[:, 1]] = np.arange(b.shape[0])
    if np.any(ids < 0):
        raise ValueError("the blocks must tile the unit cube")
    lab = ghost_lab_coords()                              # (NG, 3)
    g = b[:, None, 1:4] * BS + lab[None, :, :]            # global cell (x, y, z), (nb, NG, 3)
    g %= m * BS                                           # periodic
    nbr = g // BS
    loc = g % BS
    src_block = ids[nbr[..., 2], nbr[..., 1], nbr[..., 0]].reshape(-1).astype(np.int32)
    src_cell = (loc[..., 0] + BS * (loc[..., 1] + BS * loc[..., 2])).reshape(-1).astype(np.int32)
    n = src_block.size
    return (np.arange(n + 1, dtype=np.int64), src_block, src_cell, np.ones(n))
