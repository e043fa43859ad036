"""Test infrastructure only: ctypes binding of oracle/liboracle.so (the C
restatement in gliomauq_oracle.c). Used by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg as the checker and the timed CPU port."""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
_lib = None


def build():
    subprocess.run(["make", "-C", HERE, "lib"], check=True, stdout=subprocess.DEVNULL)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        dp = C.POINTER(C.c_double)
        fp = C.POINTER(C.c_float)
        L.orc_rd_step_f64.argtypes = [C.c_int, dp, dp, dp, dp, C.c_double, C.c_double, C.c_double,
                                      C.c_double, C.c_double, C.c_int]
        L.orc_rd_step_f32ref.argtypes = [C.c_int, fp, fp, fp, fp, C.c_float, C.c_float, C.c_float,
                                         C.c_double, C.c_double, C.c_int]
        L.orc_rd_solve_f64.argtypes = [C.c_int, dp, dp, dp, C.c_double, C.c_double, C.c_double,
                                       C.c_double, C.c_double, C.c_long, C.c_int]
        L.orc_rd_solve_f32ref.argtypes = [C.c_int, fp, fp, fp, C.c_float, C.c_float, C.c_float,
                                          C.c_double, C.c_double, C.c_long, C.c_int]
        L.orc_blockgrid_create.restype = C.c_void_p
        L.orc_blockgrid_create.argtypes = [C.c_int, fp, fp, fp]
        L.orc_blockgrid_steps.argtypes = [C.c_void_p, C.c_float, C.c_float, C.c_float, C.c_double,
                                          C.c_double, C.c_long, C.c_int]
        L.orc_blockgrid_get_phi.argtypes = [C.c_void_p, fp]
        L.orc_blockgrid_destroy.argtypes = [C.c_void_p]
        L.orc_loglik.argtypes = [C.c_int, C.c_int, C.c_int, dp, dp, dp, dp, dp, C.c_long,
                                 C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p]
        L.orc_mala_step_f64.argtypes = [C.c_int, dp, dp, dp, dp, dp, dp, dp, dp, C.c_double,
                                        C.c_double, C.c_double, C.c_double, C.c_double]
        L.orc_mala_step_f32ref.argtypes = [C.c_int, fp, fp, fp, fp, fp, fp, fp, fp, C.c_float,
                                           C.c_float, C.c_float, C.c_double, C.c_double]
        L.orc_num_steps.restype = C.c_long
        L.orc_num_steps.argtypes = [C.c_double, C.c_double]
        _lib = L
    return _lib


class LikParams(C.Structure):
    _fields_ = [("pet_sigma2", C.c_double), ("pet_scale", C.c_double), ("t1_uc", C.c_double),
                ("t2_uc", C.c_double), ("slope", C.c_double)]


class LikResult(C.Structure):
    _fields_ = [("l_pet", C.c_double), ("l_t1", C.c_double), ("l_t2", C.c_double),
                ("total", C.c_double), ("n_pet", C.c_long)]


def _p(a, t):
    return a.ctypes.data_as(C.POINTER(t))


def rd_solve(pw, pg, phi0, Dw, Dg, rho, dt, nsteps, prec="f64", nthreads=0):
    """nsteps reference steps on a uniform periodic grid; returns the final field."""
    n = pw.shape[0]
    h = 1.0 / n
    if prec == "f64":
        a = [np.ascontiguousarray(x, dtype=np.float64) for x in (pw, pg)]
        phi = np.array(phi0, dtype=np.float64, order="C", copy=True)
        lib().orc_rd_solve_f64(n, _p(a[0], C.c_double), _p(a[1], C.c_double),
                               _p(phi, C.c_double), Dw, Dg, rho, dt, h, nsteps, nthreads)
    elif prec == "f32ref":
        a = [np.ascontiguousarray(x, dtype=np.float32) for x in (pw, pg)]
        phi = np.array(phi0, dtype=np.float32, order="C", copy=True)
        lib().orc_rd_solve_f32ref(n, _p(a[0], C.c_float), _p(a[1], C.c_float),
                                  _p(phi, C.c_float), np.float32(Dw), np.float32(Dg),
                                  np.float32(rho), dt, h, nsteps, nthreads)
    else:
        raise ValueError(prec)
    return phi


def mala_solve(pw, pg, phi0, Dw, Dg, rho, dt, nsteps, prec="f64", sr0=None, sd0=None):
    """nsteps steps of the MALA variant (phi and the slopes sRho, sD, from
    zero slopes unless given); returns (phi, sRho, sD)."""
    n = pw.shape[0]
    h = 1.0 / n
    t = np.float64 if prec == "f64" else np.float32
    ct = C.c_double if prec == "f64" else C.c_float
    if prec not in ("f64", "f32ref"):
        raise ValueError(prec)
    a = [np.ascontiguousarray(x, dtype=t) for x in (pw, pg)]
    cur = [np.array(phi0, dtype=t, order="C", copy=True),
           np.zeros_like(a[0]) if sr0 is None else np.array(sr0, dtype=t, order="C", copy=True),
           np.zeros_like(a[0]) if sd0 is None else np.array(sd0, dtype=t, order="C", copy=True)]
    nxt = [np.empty_like(x) for x in cur]
    f = lib().orc_mala_step_f64 if prec == "f64" else lib().orc_mala_step_f32ref
    par = (Dw, Dg, rho) if prec == "f64" else (np.float32(Dw), np.float32(Dg), np.float32(rho))
    for _ in range(nsteps):
        f(n, _p(a[0], ct), _p(a[1], ct), *[_p(x, ct) for x in cur], *[_p(x, ct) for x in nxt],
          *par, dt, h)
        cur, nxt = nxt, cur
    return tuple(cur)


class BlockGrid:
    """The block-lab restatement of the reference's CPU step (timed baseline)."""

    def __init__(self, pw, pg, phi):
        self.n = pw.shape[0]
        a = [np.ascontiguousarray(x, dtype=np.float32) for x in (pw, pg, phi)]
        self._h = lib().orc_blockgrid_create(self.n, *[_p(x, C.c_float) for x in a])
        if not self._h:
            raise ValueError("n must be a multiple of 16")

    def steps(self, Dw, Dg, rho, dt, nsteps, nthreads=0):
        lib().orc_blockgrid_steps(self._h, np.float32(Dw), np.float32(Dg), np.float32(rho), dt,
                                  1.0 / self.n, nsteps, nthreads)

    def phi(self):
        out = np.empty((self.n,) * 3, dtype=np.float32)
        lib().orc_blockgrid_get_phi(self._h, _p(out, C.c_float))
        return out

    def __del__(self):
        if getattr(self, "_h", None):
            lib().orc_blockgrid_destroy(self._h)
            self._h = None


def loglik(model, pet, t1, t2, points, params, step_pet=3, step_ti=2, selective=True):
    """HGG_Likelihood restated; returns dict of l_pet, l_t1, l_t2, total, n_pet."""
    nz, ny, nx = model.shape
    arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (model, pet, t1, t2)]
    pts = np.ascontiguousarray(np.asarray(points, dtype=np.float64).T)  # column-major D2D
    npts = pts.shape[1] if pts.size else 0
    lp = LikParams(*params)
    res = LikResult()
    lib().orc_loglik(nx, ny, nz, *[_p(a, C.c_double) for a in arrs],
                     _p(pts, C.c_double) if npts else None, npts, C.byref(lp), step_pet, step_ti,
                     1 if selective else 0, C.byref(res))
    return dict(l_pet=res.l_pet, l_t1=res.l_t1, l_t2=res.l_t2, total=res.total, n_pet=res.n_pet)


def propagation_stats(fields, reference_rules=True):
    """Per-cell mean and variance of S density fields [S, z, y, x] as the
    reference's propagation tool forms them in Real = float
    (source/Glioma/Glioma_HG_Propagation.cpp:346-440: the sum over samples,
    then the squared deviations from inSamples * sum; then
    Glioma_PropagationStatisticsOperator.h:34-47 scales both by inSamples).
    A field value enters as the double it was stored as, so each sum step is a
    double addition rounded to float. With reference_rules, cells with a zero
    x, y or z index stay 0 (the tool's mapped-index test `> 0 && <= size`,
    :380-381 and :430). Returns two float32 [z, y, x] arrays."""
    F = np.asarray(fields, dtype=np.float32)
    S, n = F.shape[0], F.shape[1]
    inv = np.float32(1.0 / S)
    m = np.zeros(F.shape[1:], np.float32)
    for s in range(S):
        m = (m.astype(np.float64) + F[s].astype(np.float64)).astype(np.float32)
    p = (inv * m).astype(np.float32)
    v = np.zeros_like(m)
    for s in range(S):
        t = (F[s].astype(np.float64) - p.astype(np.float64)).astype(np.float32)
        v = (v + (t * t).astype(np.float32)).astype(np.float32)
    mean, var = (m * inv).astype(np.float32), (v * inv).astype(np.float32)
    if reference_rules:
        for a in (mean, var):
            a[0, :, :] = 0
            a[:, 0, :] = 0
            a[:, :, 0] = 0
    return mean, var


DRAND48_A = 0x5DEECE66D
DRAND48_C = 0xB
# drand48's state in a program that never seeds it: zero with glibc (POSIX
# leaves it unspecified; other C libraries start at 0x1234ABCD330E)
DRAND48_UNSEEDED = 0
_M48 = (1 << 48) - 1


def synthetic_observations(tumor, block_order, uc_t1=0.8, uc_t2=0.3, alpha=0.02, seed=DRAND48_UNSEEDED):
    """Synthetic PET/T1/T2 observations from a tumour density as the
    reference's Glioma_ProcessSyntheticData does them in Real = float
    (source/Glioma/Glioma_ProcessSyntheticData.cpp): _ic (:61-104, PET = the
    density where it is >= uc_t2 else 0, T1/T2 = density >= uc_t1 / uc_t2),
    then run() (:406-430): _getPETstatistic (:107-153: max, and the centre of
    mass summed in float in the grid's loop order), _normalizePETsignal
    (:156-173), _addNoise (:176-221: drand48 pairs through Box-Muller, a new
    pair at every cell while the count of noised cells is even, the first
    value to a noised cell, the second kept for the next), statistics,
    normalisation. tumor: [z, y, x] array (n = 16 * 2^l); block_order: the
    grid's blocks (level, ix, iy, iz) in the order its loops visit them.
    Returns (PET, T1, T2 as float64 arrays of the float values, centre of
    mass as 3 float32)."""
    import math
    f32 = np.float32
    t = np.asarray(tumor)
    n = t.shape[0]
    pet = t.astype(np.float32)
    phi = np.where(pet >= f32(uc_t2), pet, f32(0)).astype(np.float32).reshape(-1)
    t1 = (pet >= f32(uc_t1)).astype(np.float64)
    t2 = (pet >= f32(uc_t2)).astype(np.float64)
    # cell indices and x, y, z positions (float, as BlockInfo::pos) in loop order
    cells, pos = [], []
    for (lv, bx, by, bz) in np.asarray(block_order, dtype=np.int64):
        hf = f32(2.0 ** -int(lv) / 16)
        org = [f32(b * 2.0 ** -int(lv)) for b in (bx, by, bz)]
        z, y, x = np.meshgrid(np.arange(16), np.arange(16), np.arange(16), indexing="ij")
        gx, gy, gz = 16 * bx + x.ravel(), 16 * by + y.ravel(), 16 * bz + z.ravel()
        cells.append(gx + n * (gy + n * gz))
        pos.append(np.stack([(org[0] + hf * x.ravel().astype(np.float32)).astype(np.float32),
                             (org[1] + hf * y.ravel().astype(np.float32)).astype(np.float32),
                             (org[2] + hf * z.ravel().astype(np.float32)).astype(np.float32)], axis=1))
    cells = np.concatenate(cells)
    pos = np.concatenate(pos).astype(np.float64)

    def statistic():
        mx = f32(0)
        mass, c = f32(0), [f32(0)] * 3
        for k in np.flatnonzero(phi[cells] != 0):
            p = phi[cells[k]]
            mx = max(mx, p)
            mass = f32(mass + p)
            c = [f32(float(c[j]) + pos[k, j] * float(p)) for j in range(3)]
        return mx, np.array([f32(cj / mass) for cj in c], dtype=np.float32)

    def normalize(mx):
        iscale = 1.0 / float(mx)
        phi[:] = (phi.astype(np.float64) * iscale).astype(np.float32)

    mx, com = statistic()
    normalize(mx)
    state, ncount, xi1, xi2 = seed, 0, 0.0, 0.0

    def drand48():
        nonlocal state
        state = (DRAND48_A * state + DRAND48_C) & _M48
        return state / float(1 << 48)

    for c in cells:
        if ncount % 2 == 0:
            u1, u2 = drand48(), drand48()
            r = math.sqrt(-2.0 * math.log(u1))
            xi1 = r * math.cos(2.0 * math.pi * u2)
            xi2 = r * math.sin(2.0 * math.pi * u2)
        if phi[c] > 0:
            v = float(phi[c]) + alpha * xi1
            phi[c] = f32(v if 0.0 < v else 0.0)
            xi1 = xi2
            ncount += 1
    mx, com = statistic()
    normalize(mx)
    shape = (n, n, n)
    return phi.reshape(shape).astype(np.float64), t1, t2, com
