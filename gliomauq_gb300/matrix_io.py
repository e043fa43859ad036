"""The reference's binary matrix files (``Matrix::D2D`` / ``Matrix::D3D``).

Layout, from ``source/Glioma/Matrix.h:26-35`` and ``:609-664``: an int header
``{1234, dim, nx, ny[, nz]}``, an int type id (0 double, 1 float, 2 int), then
the elements. 3-D element (i, j, k) is at ``i + (j + k*ny)*nx``
(``Matrix.h:593-602``); 2-D element (i, j) is at ``i + j*nx``. This is the wire
format between ``brain`` and ``likelihood`` (``HGG_data.dat``, ``PET_data.dat``,
``T1_data.dat``, ``T2_data.dat``, ``Sphere.dat``) and of the anatomy files.

Arrays returned here are numpy arrays indexed ``[z, y, x]`` (3-D) or
``[j, i]`` (2-D), i.e. C order over the file's x-fastest data.
"""
from __future__ import annotations

import numpy as np

MAGIC = 1234
_TID_TO_DTYPE = {0: np.float64, 1: np.float32, 2: np.int32}
_DTYPE_TO_TID = {np.dtype(np.float64): 0, np.dtype(np.float32): 1, np.dtype(np.int32): 2}


class MatrixFormatError(ValueError):
    pass


def write_d3d(path: str, arr: np.ndarray, dtype=np.float64) -> None:
    """Write a [z, y, x] array as ``Matrix::D3D`` (default element type double)."""
    a = np.ascontiguousarray(arr, dtype=dtype)
    if a.ndim != 3:
        raise MatrixFormatError("D3D needs a 3-D array")
    nz, ny, nx = a.shape
    with open(path, "wb") as f:
        np.array([MAGIC, 3, nx, ny, nz, _DTYPE_TO_TID[a.dtype]], dtype="<i4").tofile(f)
        a.astype(a.dtype.newbyteorder("<"), copy=False).tofile(f)


def write_d2d(path: str, arr: np.ndarray, dtype=np.float64) -> None:
    """Write a [j, i] array as ``Matrix::D2D`` (nx = shape[1], ny = shape[0])."""
    a = np.ascontiguousarray(arr, dtype=dtype)
    if a.ndim != 2:
        raise MatrixFormatError("D2D needs a 2-D array")
    ny, nx = a.shape
    with open(path, "wb") as f:
        np.array([MAGIC, 2, nx, ny, _DTYPE_TO_TID[a.dtype]], dtype="<i4").tofile(f)
        a.tofile(f)


def _read(path: str, dim: int) -> np.ndarray:
    raw = np.fromfile(path, dtype=np.uint8)
    hdr_len = 4 * (2 + dim + 1)
    if raw.size < hdr_len:
        raise MatrixFormatError(f"{path}: truncated header")
    hdr = raw[:hdr_len].view("<i4")
    if hdr[0] != MAGIC:
        raise MatrixFormatError(f"{path}: magic number did not match")
    if hdr[1] != dim:
        raise MatrixFormatError(f"{path}: dimensions of matrix do not match")
    sizes = [int(s) for s in hdr[2:2 + dim]]
    if any(s < 0 for s in sizes):
        raise MatrixFormatError(f"{path}: negative size")
    tid = int(hdr[2 + dim])
    if tid not in _TID_TO_DTYPE:
        raise MatrixFormatError(f"{path}: unknown type id {tid}")
    dt = np.dtype(_TID_TO_DTYPE[tid]).newbyteorder("<")
    n = int(np.prod(sizes))
    body = raw[hdr_len:]
    if body.size < n * dt.itemsize:
        raise MatrixFormatError(f"{path}: truncated data")
    data = body[: n * dt.itemsize].view(dt).astype(np.float64)
    return data.reshape(tuple(reversed(sizes)))


def read_d3d(path: str) -> np.ndarray:
    """Read ``Matrix::D3D`` into a float64 [z, y, x] array."""
    return _read(path, 3)


def read_d2d(path: str) -> np.ndarray:
    """Read ``Matrix::D2D`` into a float64 [j, i] array."""
    return _read(path, 2)
