"""Posterior sampling of the tumour parameters over the GPU solver.

The reference leaves sampling to an external TMCMC driver that runs one
`brain` + `likelihood` process pair per sample. Here chains are advanced in
lock-step and every generation's forward solves (and, for MALA, adjoint
gradients) are one batched library call; accept/reject and all densities are
in float64 on the host.

Parameters theta = (Dw [cm^2/day], rho [1/day], x0, y0, z0 [voxel], T [day]);
uniform prior on a box for Dw, rho, T and on the interior seed region for
(x0, y0, z0). Chains move in coordinates scaled by the prior box widths.

  * rwm  : random-walk Metropolis, Gaussian proposal
  * mala : Metropolis-adjusted Langevin, gradients from gbg_adjoint_grad
  * ess  : effective sample size per parameter (Geyer's initial monotone
           sequence on the chain-averaged autocorrelation)
Both samplers use the adjoint's smooth-time-grid forward model for log L,
so they target the same posterior.
"""
from __future__ import annotations

import time
from dataclasses import dataclass, field

import numpy as np

from . import synthetic as Syn

NAMES = ("Dw", "rho", "x0", "y0", "z0", "T")


@dataclass
class Prior:
    lo: np.ndarray
    hi: np.ndarray
    seed_mask: np.ndarray  # [z, y, x] bool: allowed voxels for the seed

    @classmethod
    def from_anatomy(cls, anat: Syn.Anatomy):
        pts = Syn.seed_box_points(anat)
        lo = np.array([Syn.PRIOR_DW_CM2[0], Syn.PRIOR_RHO[0], *(pts.min(axis=0) - 0.5),
                       Syn.PRIOR_T[0]])
        hi = np.array([Syn.PRIOR_DW_CM2[1], Syn.PRIOR_RHO[1], *(pts.max(axis=0) + 0.5),
                       Syn.PRIOR_T[1]])
        mask = np.zeros(anat.brain.shape, dtype=bool)
        ix = pts.astype(int)
        mask[ix[:, 2], ix[:, 1], ix[:, 0]] = True
        return cls(lo=lo, hi=hi, seed_mask=mask)

    @property
    def width(self):
        return self.hi - self.lo

    def logp(self, theta: np.ndarray) -> np.ndarray:
        """0 inside the support, -inf outside; theta is (chains, 6)."""
        th = np.atleast_2d(theta)
        ok = np.all((th >= self.lo) & (th <= self.hi), axis=1)
        v = np.rint(th[:, 2:5]).astype(int)
        n = self.seed_mask.shape[0]
        inb = np.all((v >= 0) & (v < n), axis=1)
        v = np.clip(v, 0, n - 1)
        ok &= inb & self.seed_mask[v[:, 2], v[:, 1], v[:, 0]]
        return np.where(ok, 0.0, -np.inf)


@dataclass
class Posterior:
    """log L from the GPU solver (smooth time grid, float states)."""
    handle: object
    L: float
    dt0: float
    prior: Prior
    ic_peak: float = 0.1
    ic_sigma: float = 1.0
    checkpoint_every: int = 50
    calls: int = 0
    solves: int = 0
    seconds: float = 0.0

    def loglik(self, theta: np.ndarray, with_grad: bool):
        th = np.atleast_2d(theta)
        lp = self.prior.logp(th)
        ll = np.full(th.shape[0], -np.inf)
        g = np.zeros_like(th)
        ok = np.isfinite(lp)
        if ok.any():
            t0 = time.perf_counter()
            l, gr = self.handle.adjoint_grad([tuple(x) for x in th[ok]], self.dt0, self.L,
                                             ic_peak=self.ic_peak, ic_sigma=self.ic_sigma,
                                             checkpoint_every=self.checkpoint_every,
                                             state="f32", want_grad=with_grad)
            self.seconds += time.perf_counter() - t0
            self.calls += 1
            self.solves += int(ok.sum())
            ll[ok] = l
            if with_grad:
                g[ok] = gr
        return ll + lp, g


@dataclass
class ChainResult:
    samples: np.ndarray  # (steps, chains, 6)
    accept: float
    step: float
    seconds: float
    solves: int
    history: dict = field(default_factory=dict)


def rwm(post: Posterior, theta0: np.ndarray, steps: int, step: float, rng, burn: int = 0,
        target: float = 0.234) -> ChainResult:
    """Random-walk Metropolis in prior-width-scaled coordinates; the step is
    adapted toward the target acceptance during the first `burn` steps."""
    th = np.array(theta0, dtype=np.float64)
    lp, _ = post.loglik(th, False)
    out = np.empty((steps,) + th.shape)
    acc = 0
    t0 = time.perf_counter()
    for k in range(steps):
        prop = th + step * post.prior.width * rng.standard_normal(th.shape)
        lq, _ = post.loglik(prop, False)
        a = np.log(rng.random(th.shape[0])) < lq - lp
        th[a], lp[a] = prop[a], lq[a]
        if k < burn:
            step *= np.exp((a.mean() - target) / np.sqrt(k + 1.0))
        else:
            acc += a.sum()
        out[k] = th
    n_acc = max(1, (steps - burn) * th.shape[0])
    return ChainResult(out, acc / n_acc, step, time.perf_counter() - t0, post.solves)


def mala(post: Posterior, theta0: np.ndarray, steps: int, eps: float, rng, burn: int = 0,
         target: float = 0.574) -> ChainResult:
    """MALA in prior-width-scaled coordinates z = theta / width: proposal
    z' = z + eps^2/2 grad_z log pi + eps xi, accepted with the Metropolis-
    Hastings ratio of the two Langevin proposal densities."""
    w = post.prior.width
    th = np.array(theta0, dtype=np.float64)
    lp, g = post.loglik(th, True)
    gz = g * w
    out = np.empty((steps,) + th.shape)
    acc = 0
    t0 = time.perf_counter()
    for k in range(steps):
        xi = rng.standard_normal(th.shape)
        zp = th / w + 0.5 * eps ** 2 * gz + eps * xi
        prop = zp * w
        lq, gq = post.loglik(prop, True)
        gqz = gq * w
        fwd = -np.sum((zp - th / w - 0.5 * eps ** 2 * gz) ** 2, axis=1) / (2 * eps ** 2)
        bwd = -np.sum((th / w - zp - 0.5 * eps ** 2 * gqz) ** 2, axis=1) / (2 * eps ** 2)
        with np.errstate(invalid="ignore"):
            logr = lq - lp + bwd - fwd
        a = np.isfinite(lq) & (np.log(rng.random(th.shape[0])) < logr)
        th[a], lp[a], gz[a] = prop[a], lq[a], gqz[a]
        if k < burn:
            eps *= np.exp((a.mean() - target) / np.sqrt(k + 1.0))
        else:
            acc += a.sum()
        out[k] = th
    n_acc = max(1, (steps - burn) * th.shape[0])
    return ChainResult(out, acc / n_acc, eps, time.perf_counter() - t0, post.solves)


def _autocov(x: np.ndarray) -> np.ndarray:
    n = x.size
    f = np.fft.rfft(x - x.mean(), n=2 * n)
    ac = np.fft.irfft(f * np.conjugate(f))[:n]
    return ac / n


def ess(samples: np.ndarray) -> np.ndarray:
    """Effective sample size per parameter of (steps, chains, d) draws:
    chain-averaged autocorrelation (split-free version of the multi-chain
    estimator) with Geyer's initial monotone sequence truncation."""
    n, m, d = samples.shape
    out = np.zeros(d)
    for j in range(d):
        x = samples[:, :, j]
        acov = np.stack([_autocov(x[:, c]) for c in range(m)])
        w = acov[:, 0].mean() * n / max(n - 1, 1)
        b = n * x.mean(axis=0).var(ddof=1) if m > 1 else 0.0
        var_plus = (n - 1) / n * w + b / n
        if var_plus <= 0:
            out[j] = float(n * m)
            continue
        rho = 1.0 - (w - acov.mean(axis=0)) / var_plus
        rho[0] = 1.0
        s, prev = 0.0, np.inf
        for t in range(0, n - 1, 2):
            pair = rho[t] + rho[t + 1]
            if pair < 0:
                break
            pair = min(pair, prev)
            s += pair
            prev = pair
        tau = max(-1.0 + 2.0 * s, 1.0 / np.log10(max(n * m, 10)))
        out[j] = n * m / tau
    return out
