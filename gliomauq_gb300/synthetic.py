"""Seeded synthetic anatomy, initial densities, priors and observations.

The reference's patient and BrainWeb anatomies and its likelihood data files
are not available, so every input is generated here from
``numpy.random.default_rng(seed)`` and handed identically to the CUDA path and
to the CPU oracle. Nothing here reproduces a dataset item.

Anatomy(N), voxel spacing 1 mm:
  * ellipsoid centred at (N-1)/2 on every axis, semi-axes (28, 24, 22) * N/64
    voxels, normalised radius r;
  * phase field psi = 0.5 * (1 - tanh((r - 1) * a_min)) with a_min the smallest
    semi-axis; psi < 1e-3 is set to exactly 0, and a 4-voxel margin at every
    face is zeroed so the periodic domain keeps the brain off its faces;
  * white-matter indicator m = [g > 0] for a Gaussian random field g (white
    noise convolved with a Gaussian of sigma 4 voxels, periodic FFT);
  * p_w = psi * m, p_g = psi * (1 - m), CSF = 0.
Units follow the reference: the domain is the unit cube with brain length
L = N * 0.1 cm (``Glioma_HG_UQ.cpp:104``); Dw is given in cm^2/day as in
``HGG_InputParameters.txt`` (config values in mm^2/day divide by 100).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

SEMI_AXES_64 = (28.0, 24.0, 22.0)
MARGIN = 4
GRF_SIGMA = 4.0


@dataclass
class Anatomy:
    n: int
    p_w: np.ndarray  # [z, y, x] float64
    p_g: np.ndarray
    psi: np.ndarray

    @property
    def brain(self) -> np.ndarray:
        return (self.p_w + self.p_g) > 0

    @property
    def L(self) -> float:
        """Brain length in cm, as ``L = brainSizeMax * 0.1`` (Glioma_HG_UQ.cpp:104)."""
        return self.n * 0.1


def _radius(n: int) -> np.ndarray:
    c = (n - 1) / 2.0
    a = [s * n / 64.0 for s in SEMI_AXES_64]
    z, y, x = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    return np.sqrt(((x - c) / a[0]) ** 2 + ((y - c) / a[1]) ** 2 + ((z - c) / a[2]) ** 2)


def make_anatomy(n: int, seed: int = 0) -> Anatomy:
    rng = np.random.default_rng(seed)
    r = _radius(n)
    a_min = min(SEMI_AXES_64) * n / 64.0
    psi = 0.5 * (1.0 - np.tanh((r - 1.0) * a_min))
    psi[psi < 1e-3] = 0.0
    psi[:MARGIN, :, :] = psi[-MARGIN:, :, :] = 0.0
    psi[:, :MARGIN, :] = psi[:, -MARGIN:, :] = 0.0
    psi[:, :, :MARGIN] = psi[:, :, -MARGIN:] = 0.0
    white = rng.standard_normal((n, n, n))
    k = np.fft.fftfreq(n)
    kz, ky, kx = np.meshgrid(k, k, k, indexing="ij")
    kern = np.exp(-2.0 * (np.pi * GRF_SIGMA) ** 2 * (kx ** 2 + ky ** 2 + kz ** 2))
    g = np.real(np.fft.ifftn(np.fft.fftn(white) * kern))
    m = (g > 0).astype(np.float64)
    return Anatomy(n=n, p_w=psi * m, p_g=psi * (1.0 - m), psi=psi)


def seed_box_points(anat: Anatomy) -> np.ndarray:
    """Voxel centres with normalised ellipsoid radius < 0.6 (the interior seed box)."""
    r = _radius(anat.n)
    z, y, x = np.nonzero((r < 0.6) & anat.brain)
    return np.stack([x, y, z], axis=1).astype(np.float64)


def gaussian_ic(anat: Anatomy, x0: float, y0: float, z0: float,
                peak: float = 0.1, sigma: float = 1.0) -> np.ndarray:
    """phi0 = peak * exp(-|x - x0|^2 / (2 sigma^2)) in voxel units, zero outside tissue."""
    n = anat.n
    z, y, x = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    d2 = (x - x0) ** 2 + (y - y0) ** 2 + (z - z0) ** 2
    phi = peak * np.exp(-d2 / (2.0 * sigma * sigma))
    phi[~anat.brain] = 0.0
    return phi


@dataclass
class SampleParams:
    """One forward solve: Dw in cm^2/day, rho in 1/day, seed in voxel units, T in days."""
    Dw: float
    rho: float
    x0: float
    y0: float
    z0: float
    T: float

    def as_tuple(self):
        return (self.Dw, self.rho, self.x0, self.y0, self.z0, self.T)


# Uniform priors: Dw 0.02..0.25 mm^2/day (0.0002..0.0025 cm^2/day),
# rho 0.01..0.2 /day, T 100..500 days, seed in the interior seed box.
PRIOR_DW_CM2 = (0.02 / 100.0, 0.25 / 100.0)
PRIOR_RHO = (0.01, 0.2)
PRIOR_T = (100.0, 500.0)


def draw_prior(anat: Anatomy, count: int, seed: int) -> list[SampleParams]:
    rng = np.random.default_rng(seed)
    pts = seed_box_points(anat)
    out = []
    for _ in range(count):
        p = pts[rng.integers(len(pts))] + rng.uniform(-0.5, 0.5, size=3)
        out.append(SampleParams(
            Dw=float(rng.uniform(*PRIOR_DW_CM2)), rho=float(rng.uniform(*PRIOR_RHO)),
            x0=float(p[0]), y0=float(p[1]), z0=float(p[2]), T=float(rng.uniform(*PRIOR_T))))
    return out


def reference_dt(n: int, Dw_cm2: float, L: float | None = None, f32: bool = False) -> tuple:
    """dt and unit-cube (Dw, Dg) exactly as Glioma_HG_UQ::run computes them
    (Glioma_HG_UQ.cpp:532-539): Dw /= L^2; Dg = 0.1*Dw; h = 1/n;
    dt = 0.99*h*h/(2*3*max(Dw, Dg)). With f32=True, Dw and Dg are rounded to
    float at each assignment as the default (Real=float) build does."""
    if L is None:
        L = n * 0.1
    if f32:
        Dw = np.float32(np.float64(np.float32(Dw_cm2)) / (L * L))
        Dg = np.float32(0.1 * np.float64(Dw))
        dw64, dg64 = float(Dw), float(Dg)
    else:
        dw64 = Dw_cm2 / (L * L)
        dg64 = 0.1 * dw64
    h = 1.0 / n
    dt = 0.99 * h * h / (2.0 * 3 * max(dw64, dg64))
    return dt, dw64, dg64


def num_steps(dt: float, tend: float) -> int:
    """Steps of ``while (t <= tend) t += dt`` (Glioma_HG_UQ.cpp:544-552)."""
    t = 0.0
    k = 0
    while t <= tend:
        t += dt
        k += 1
    return k


@dataclass
class Observations:
    pet: np.ndarray  # [z, y, x] float64
    t1: np.ndarray   # 0/1 float64
    t2: np.ndarray
    points: np.ndarray  # (npoints, 3) voxel indices (x, y, z) as float64


def make_observations(u_true: np.ndarray, anat: Anatomy, seed: int,
                      centre_xyz, radius_vox: float = 27.0,
                      flip: float = 0.05, pet_sd: float = 0.05) -> Observations:
    """T1 = [u > 0.7], T2 = [u > 0.25] with independent 5% label flips; PET =
    max(0, u + N(0, 0.05^2)) where u > 0, else 0; the selective point set is
    the tissue voxels within radius_vox of centre (the reference's 0.21-unit
    sphere rule, Glioma_HG_UQ.cpp:450-476)."""
    rng = np.random.default_rng(seed)
    t1 = (u_true > 0.7).astype(np.float64)
    t2 = (u_true > 0.25).astype(np.float64)
    f1 = rng.random(u_true.shape) < flip
    f2 = rng.random(u_true.shape) < flip
    t1[f1] = 1.0 - t1[f1]
    t2[f2] = 1.0 - t2[f2]
    noise = rng.normal(0.0, pet_sd, size=u_true.shape)
    pet = np.where(u_true > 0, np.maximum(0.0, u_true + noise), 0.0)
    n = anat.n
    z, y, x = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    cx, cy, cz = centre_xyz
    d = np.sqrt((x - cx) ** 2 + (y - cy) ** 2 + (z - cz) ** 2)
    sel = (d <= radius_vox) & anat.brain
    # same traversal order as _dumpSubBrainPoints: block by block there; here
    # z, y, x order (the order only changes the summation order of the T terms)
    zz, yy, xx = np.nonzero(sel)
    pts = np.stack([xx, yy, zz], axis=1).astype(np.float64)
    return Observations(pet=pet, t1=t1, t2=t2, points=pts)
