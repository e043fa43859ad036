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
  * tmcmc: transitional MCMC (Ching & Chen 2007), the population sampler
           of the reference's workflow, every Metropolis step of the
           population one batched solve
  * plain_chains: single-solve chains, the plain method
  * da   : delayed acceptance (Christen & Fox 2005) in its surrogate-
           transition form (Liu 2001, sec. 9.4): stage 1 runs `inner`
           random-walk Metropolis steps on the learned surrogate's
           posterior pi*, stage 2 accepts the end point y of that chain
           with min(1, pi(y) pi*(x) / (pi(x) pi*(y))), pi from the solver.
           The inner chain is reversible with respect to pi*, so the
           composite kernel is reversible with respect to pi: the solver
           judges every accepted sample and the chain targets the exact
           posterior whatever the surrogate's error.
  * ess  : effective sample size per parameter (Geyer's initial monotone
           sequence on the chain-averaged autocorrelation)
All samplers use the adjoint's smooth-time-grid forward model for log L,
so they target the same posterior. Log densities and accept/reject are
float64 throughout.
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
        """log posterior (and its gradient) of each row of theta. Without the
        gradient, log L comes from the batched population solver on the same
        smooth time grid (bitwise the adjoint's forward model), in chunks of
        the handle's max_samples."""
        th = np.atleast_2d(theta)
        lp = self.prior.logp(th)
        ll = np.full(th.shape[0], -np.inf)
        g = np.zeros_like(th)
        ok = np.isfinite(lp)
        if ok.any():
            t0 = time.perf_counter()
            rows = [tuple(x) for x in th[ok]]
            if with_grad:
                l, gr = self.handle.adjoint_grad(rows, self.dt0, self.L, ic_peak=self.ic_peak,
                                                 ic_sigma=self.ic_sigma,
                                                 checkpoint_every=self.checkpoint_every,
                                                 state="f32", want_grad=True)
                g[ok] = gr
                self.calls += 1
            else:
                cap = max(1, self.handle.max_samples)
                l = np.empty(len(rows))
                for s0 in range(0, len(rows), cap):
                    r = self.handle.batch_solve(rows[s0:s0 + cap], self.L, ic_peak=self.ic_peak,
                                                ic_sigma=self.ic_sigma, dt0=self.dt0)
                    l[s0:s0 + cap] = [d["total"] for d in r["loglik"]]
                    self.calls += 1
            self.seconds += time.perf_counter() - t0
            self.solves += int(ok.sum())
            ll[ok] = l
        return ll + lp, g


@dataclass
class ChainResult:
    samples: np.ndarray  # (steps, chains, 6)
    accept: float
    step: float
    seconds: float
    solves: int
    history: dict = field(default_factory=dict)


def _chol(post, chol):
    """Proposal scale: a Cholesky factor in parameter units (default: the
    prior box widths on the diagonal)."""
    return np.diag(post.prior.width) if chol is None else np.asarray(chol, dtype=np.float64)


def rwm(post: Posterior, theta0: np.ndarray, steps: int, step: float, rng, burn: int = 0,
        target: float = 0.234, chol=None) -> ChainResult:
    """Random-walk Metropolis with proposal theta + step * chol xi (chol
    defaults to the prior widths); the step is adapted toward the target
    acceptance during the first `burn` steps."""
    th = np.array(theta0, dtype=np.float64)
    Lc = _chol(post, chol)
    lp, _ = post.loglik(th, False)
    out = np.empty((steps,) + th.shape)
    acc = 0
    t0 = time.perf_counter()
    for k in range(steps):
        prop = th + step * rng.standard_normal(th.shape) @ Lc.T
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
         target: float = 0.574, chol=None) -> ChainResult:
    """Preconditioned MALA with metric M = chol chol^T (default: the prior
    widths squared): theta' = theta + eps^2/2 M grad log pi + eps chol xi,
    accepted with the Metropolis-Hastings ratio of the two Langevin proposal
    densities (Gaussians of covariance eps^2 M)."""
    th = np.array(theta0, dtype=np.float64)
    Lc = _chol(post, chol)
    M = Lc @ Lc.T
    Li = np.linalg.inv(Lc)
    lp, g = post.loglik(th, True)
    out = np.empty((steps,) + th.shape)
    acc = 0
    t0 = time.perf_counter()
    for k in range(steps):
        xi = rng.standard_normal(th.shape)
        mean_f = th + 0.5 * eps ** 2 * g @ M
        prop = mean_f + eps * xi @ Lc.T
        lq, gq = post.loglik(prop, True)
        mean_b = prop + 0.5 * eps ** 2 * gq @ M
        fwd = -np.sum(((prop - mean_f) @ Li.T) ** 2, axis=1) / (2 * eps ** 2)
        bwd = -np.sum(((th - mean_b) @ Li.T) ** 2, axis=1) / (2 * eps ** 2)
        with np.errstate(invalid="ignore"):
            logr = lq - lp + bwd - fwd
        a = np.isfinite(lq) & (np.log(rng.random(th.shape[0])) < logr)
        th[a], lp[a], g[a] = prop[a], lq[a], gq[a]
        if k < burn:
            eps *= np.exp((a.mean() - target) / np.sqrt(k + 1.0))
        else:
            acc += a.sum()
        out[k] = th
    n_acc = max(1, (steps - burn) * th.shape[0])
    return ChainResult(out, acc / n_acc, eps, time.perf_counter() - t0, post.solves)


def plain_chains(post, v0: np.ndarray, steps: int, cov: np.ndarray, rng, burn: int = 0,
                 axis: int = 0, step: float = None, target: float = 0.25) -> ChainResult:
    """Plain single-solve MCMC: every chain (row of v0, coordinates of a
    LogCoords posterior) runs on its own, one forward solve per step, the
    chains one after another. The proposal is the random walk
    v' = v + step * C xi on the coordinates other than `axis` (C C^T = cov
    with `axis` decoupled: the Laplace-preconditioned proposal), with v'_axis
    drawn from the prior conditional given the others (prior.redraw_axis);
    accepted with min(1, L(v') m(v') / (L(v) m(v))), m the prior marginal
    of the other coordinates (prior.axis_log_marginal), which is the
    Metropolis-Hastings ratio of this proposal for pi = L * prior. The step
    is adapted toward `target` during the first `burn` steps of each chain
    and fixed after them."""
    v0 = np.atleast_2d(np.asarray(v0, dtype=np.float64))
    m, d = v0.shape
    Lc = np.linalg.cholesky(_decoupled(np.asarray(cov, dtype=np.float64), axis))
    step0 = 2.38 / np.sqrt(d - 1) if step is None else step
    pr = post.prior
    out = np.empty((steps, m, d))
    acc = 0
    steps_used = []
    t0 = time.perf_counter()
    t_burn = 0.0
    for c in range(m):
        v = v0[c:c + 1].copy()
        lp, _ = post.loglik(v, False)
        ll = lp - pr.logp(v) + pr.axis_log_marginal(v, axis)
        st = step0
        tb = time.perf_counter()
        for k in range(steps):
            if k == burn:
                t_burn += time.perf_counter() - tb
            prop = v + st * rng.standard_normal((1, d)) @ Lc.T
            prop[:, axis] = v[:, axis]
            prop = pr.redraw_axis(prop, axis, rng)
            lm = pr.axis_log_marginal(prop, axis)
            if np.isfinite(lm[0]):
                lq, _ = post.loglik(prop, False)
                lq = lq - pr.logp(prop) + lm
            else:
                lq = lm
            with np.errstate(invalid="ignore"):
                a = bool(np.isfinite(lq[0]) and np.log(rng.random()) < lq[0] - ll[0])
            if a:
                v, ll = prop, lq
            if k < burn:
                st *= np.exp((float(a) - target) / np.sqrt(k + 1.0))
            else:
                acc += int(a)
            out[k, c] = v[0]
        if burn >= steps:
            t_burn += time.perf_counter() - tb
        steps_used.append(st)
    n_acc = max(1, (steps - burn) * m)
    return ChainResult(out, acc / n_acc, float(np.mean(steps_used)), time.perf_counter() - t0,
                       post.solves, history=dict(burn_seconds=t_burn, steps=steps_used))


@dataclass
class SurrogatePosterior:
    """log pi*(theta) = the surrogate's predicted log L + log prior, in
    batches of the surrogate's batch_max."""
    surrogate: object
    prior: Prior
    calls: int = 0
    evals: int = 0
    seconds: float = 0.0

    def logpost(self, theta: np.ndarray) -> np.ndarray:
        th = np.atleast_2d(theta)
        lp = self.prior.logp(th)
        out = np.full(th.shape[0], -np.inf)
        idx = np.nonzero(np.isfinite(lp))[0]
        bm = self.surrogate.batch_max
        t0 = time.perf_counter()
        for s0 in range(0, idx.size, bm):
            sl = idx[s0:s0 + bm]
            r = self.surrogate.loglik([tuple(x) for x in th[sl]])["loglik"]
            out[sl] = [d["total"] for d in r]
            self.calls += 1
        self.evals += idx.size
        self.seconds += time.perf_counter() - t0
        return out + lp


def _chol_population(th: np.ndarray, w: np.ndarray) -> np.ndarray:
    """Cholesky factor of the chains' covariance, in parameter units,
    normalised so that its mean variance in prior-width-scaled coordinates is
    one (its shape, not its size)."""
    d = th.shape[1]
    c = np.cov(th / w, rowvar=False) if th.shape[0] > d else np.eye(d)
    c = c / max(np.trace(c) / d, 1e-300) + 1e-6 * np.eye(d)
    return np.diag(w) @ np.linalg.cholesky(c)


def _decoupled(c: np.ndarray, axis) -> np.ndarray:
    """Covariance with coordinate `axis` made independent of the others (its
    own variance kept): random-walk moves of the other coordinates then use
    their marginal covariance."""
    if axis is None:
        return c
    c = np.array(c, dtype=np.float64, copy=True)
    var = c[axis, axis]
    c[axis, :] = 0.0
    c[:, axis] = 0.0
    c[axis, axis] = var if var > 0 else 1.0
    return c


def _chol_cov(th: np.ndarray, axis=None) -> np.ndarray:
    """Cholesky factor of the chains' covariance in parameter units."""
    c = _decoupled(np.cov(th, rowvar=False), axis)
    return np.linalg.cholesky(c + 1e-12 * np.diag(np.diag(c)) + 1e-300 * np.eye(c.shape[0]))


STRANDED_NATS = 25.0  # a chain this far below the population's median log pi is stranded


def _stranded(lp: np.ndarray) -> np.ndarray:
    """Chains whose log pi is not finite or lies more than STRANDED_NATS below
    the population median (far outside the bulk of a posterior with a few
    identified parameters: chi^2_5 / 2 exceeds 10.3 with probability 1e-3)."""
    ok = np.isfinite(lp)
    if not ok.any():
        return ~ok
    return ~ok | (lp < np.median(lp[ok]) - STRANDED_NATS)


def _discrepancy(lp: np.ndarray, ls: np.ndarray) -> float:
    """Spread of log pi - log pi_surrogate over the population: what the
    second stage's acceptance depends on (a constant offset cancels)."""
    ok = np.isfinite(lp) & np.isfinite(ls)
    return float(np.std(lp[ok] - ls[ok])) if ok.sum() >= 3 else np.inf


def inner_chain(prior, spost, y: np.ndarray, ly: np.ndarray, steps: int, step: float, Lc: np.ndarray,
                axis, axis_prob: float, rng, ind=None):
    """da's first stage on the host: `steps` Metropolis steps on the
    surrogate posterior for every row of y (log densities ly): with `axis`
    set, each step is with probability axis_prob a redraw of that coordinate
    from its prior conditional (prior.redraw_axis; an independence proposal
    whose prior factors cancel, leaving the surrogate's likelihood ratio);
    with ind = (probability, mean, factor G, axis decoupled) an independence
    proposal mean + G xi for the other coordinates, accepted with the ratio
    of that Gaussian's densities; otherwise the random walk y + step * Lc xi
    on the other coordinates. Returns (end points, their log densities,
    random-walk acceptances, random-walk steps)."""
    y, ly = np.array(y, dtype=np.float64, copy=True), np.array(ly, dtype=np.float64, copy=True)
    m, d = y.shape
    ip, im, ig = (0.0, None, None) if ind is None else ind
    gi = np.linalg.inv(ig) if ip > 0 else None
    ident = np.ones(d, dtype=bool)
    if axis is not None:
        ident[axis] = False
    na = nt = 0
    for _ in range(steps):
        xi = rng.standard_normal((m, d))
        prop = y + step * xi @ Lc.T
        corr = np.zeros(m)
        jump = np.zeros(m, dtype=bool)
        u = rng.random(m)
        if axis is not None:
            prop[:, axis] = y[:, axis]
            jump = u < axis_prob
            if jump.any():
                prop[jump] = prior.redraw_axis(y[jump], axis, rng)
                corr[jump] = prior.logp(y[jump]) - prior.logp(prop[jump])
        indep = ~jump & (u < (axis_prob if axis is not None else 0.0) + ip)
        if indep.any():
            z = xi[indep] * ident
            prop[indep] = np.where(ident, im + z @ ig.T, y[indep])
            zv = ((y[indep] - im) @ gi.T) * ident
            corr[indep] = 0.5 * (np.sum(z * z, axis=1) - np.sum(zv * zv, axis=1))
        lq = spost.logpost(prop)
        with np.errstate(invalid="ignore"):
            a = np.isfinite(lq) & (np.log(rng.random(m)) < lq - ly + corr)
        y[a], ly[a] = prop[a], lq[a]
        rwm = ~jump & ~indep
        na += int(a[rwm].sum())
        nt += int(rwm.sum())
    return y, ly, na, nt


def da(post: Posterior, spost: SurrogatePosterior, theta0: np.ndarray, steps: int, step: float,
       rng, inner: int = 8, burn: int = 0, target: float = 0.3, chol=None, adapt: bool = False,
       rebuild_every: int = 0, axis=None, axis_prob: float = 0.5,
       adapt_pool: bool = True, reset_stranded: bool = True, gpu_chain: bool = True,
       ind_prob: float = 0.0, ind_scale: float = 1.2) -> ChainResult:
    """Delayed-acceptance MCMC, chains in lock-step: per generation `inner`
    batched surrogate calls and one batched solver call for the chains whose
    inner chain moved. The inner random-walk proposal is y + step * C xi:
    C = chol if given, else the prior widths. During the first `burn`
    generations the step is adapted toward the target inner acceptance and,
    with adapt=True (or chol None), C follows the population covariance of
    the chains (adapt_pool: pooled over the chains and the latter half of the
    generations so far, a far steadier estimate than one generation's
    `chains` points, stranded chain-generations left out); every
    `rebuild_every` burn-in generations a surrogate that has
    rebuild(u_centre, steps) is re-linearised at the population median with
    half the population standard deviations as steps, and kept only if it
    lowers the spread of log pi - log pi_surrogate over the population
    (state()/restore() put the previous build back otherwise). With
    reset_stranded, chains stranded far below the population (_stranded) are
    moved to copies of randomly chosen other chains at those points and once
    more when burn-in ends; burn-in output is discarded, so this only
    changes where the fixed post-burn-in kernel starts. With `axis` = a
    (the scaling symmetry's coordinate in the invariant coordinates, along
    which the likelihood of the scaled time grid is flat), random-walk moves
    leave coordinate a fixed and each inner step is, with probability
    axis_prob, instead a redraw of coordinate a from its prior conditional
    (post.prior.redraw_axis), an independence proposal accepted with the
    ratio of the surrogate's likelihoods (its prior terms cancel the
    proposal's). Both moves keep the inner chain reversible with respect to
    the surrogate posterior. All of it is frozen after burn-in, so the
    sampled chain is a fixed reversible kernel whose invariant law is the
    exact posterior. With gpu_chain and a surrogate that has chain() (the
    affine screen), each generation's inner chains run on the GPU in one
    launch (the same moves, device random numbers), which also returns the
    screen's log density at the chains' current points for stage 2. With
    ind_prob > 0 an inner step is, with that probability, an independence
    proposal from a Gaussian on the coordinates other than `axis`: the
    population's (pooled) mean and covariance inflated by ind_scale, adapted
    with the random-walk covariance during burn-in and frozen after it."""
    w = post.prior.width
    th = np.array(theta0, dtype=np.float64)
    m, d = th.shape
    lp, _ = post.loglik(th, False)
    ls = spost.logpost(th)
    Lc = _chol(post, chol)
    if axis is not None:
        Lc = np.linalg.cholesky(_decoupled(Lc @ Lc.T, axis))
    ind_mean, ind_G = np.median(th, axis=0), ind_scale * Lc
    out = np.empty((steps, m, d))
    lp_out = np.empty((steps, m))
    acc1 = acc2 = tried = 0
    resets = rebuilds_kept = rebuilds_tried = 0
    t0 = time.perf_counter()
    t_burn = 0.0

    def reset():
        nonlocal resets
        bad = _stranded(lp)
        if bad.any() and not bad.all():
            src = rng.choice(np.flatnonzero(~bad), size=int(bad.sum()))
            th[bad], lp[bad], ls[bad] = th[src], lp[src], ls[src]
            resets += int(bad.sum())

    for k in range(steps):
        if k == burn:
            if reset_stranded and burn > 0:
                reset()
            t_burn = time.perf_counter() - t0
        if k < burn and m > 2 * d:
            if rebuild_every > 0 and k > 0 and k % rebuild_every == 0:
                if reset_stranded:
                    reset()
                if hasattr(spost, "rebuild"):
                    good = ~_stranded(lp)
                    old = spost.state() if hasattr(spost, "state") else None
                    spost.rebuild(np.median(th[good], axis=0), 0.5 * th[good].std(axis=0))
                    ls_new = spost.logpost(th)
                    rebuilds_tried += 1
                    if old is not None and _discrepancy(lp, ls_new) > _discrepancy(lp, ls):
                        spost.restore(old)
                    else:
                        ls = ls_new
                        rebuilds_kept += 1
            if chol is None:
                Lc = _chol_population(th, w)
            elif adapt and k >= max(1, burn // 4):
                if adapt_pool:
                    win = slice(k // 2, k)
                    keep = np.stack([~_stranded(r) for r in lp_out[win]])
                    pts = out[win][keep]
                    pts = pts if len(pts) > 2 * d else th
                else:
                    pts = th
                Lc = _chol_cov(pts, axis)
                ind_mean, ind_G = pts.mean(axis=0), ind_scale * Lc
        ind = (ind_prob, ind_mean, ind_G) if ind_prob > 0 else None
        if gpu_chain and getattr(spost, "gpu_chain_ready", False):
            # random-walk acceptance fraction a1 (the step adapts to it)
            y, ls, ly, a1 = spost.chain(th, inner, step, Lc, axis, axis_prob,
                                        int(rng.integers(0, 2 ** 63)), ind=ind)
        else:
            y, ly, na, nt = inner_chain(post.prior, spost, th, ls, inner, step, Lc, axis, axis_prob,
                                        rng, ind=ind)
            a1 = na / max(nt, 1)
        moved = np.any(y != th, axis=1)
        if moved.any():
            lpy = np.full(m, -np.inf)
            lpy[moved], _ = post.loglik(y[moved], False)
            with np.errstate(invalid="ignore"):
                logr = (lpy - lp) - (ly - ls)
            # a chain outside the support moves to any point inside it
            logr = np.where(np.isneginf(lp) & np.isfinite(lpy), np.inf, logr)
            a = moved & np.isfinite(lpy) & (np.log(rng.random(m)) < logr)
            th[a], lp[a], ls[a] = y[a], lpy[a], ly[a]
        else:
            a = np.zeros(m, dtype=bool)
        if k < burn:
            step *= np.exp((a1 - target) / np.sqrt(k + 1.0))
        else:
            acc1 += a1 * m
            acc2 += a.sum()
            tried += moved.sum()
        out[k] = th
        lp_out[k] = lp
    n_gen = max(1, (steps - burn) * m)
    return ChainResult(out, acc2 / n_gen, step, time.perf_counter() - t0, post.solves,
                       history=dict(stage1_accept=acc1 / n_gen,  # random-walk moves
                                    stage2_accept=acc2 / max(tried, 1),
                                    surrogate_evals=spost.evals, inner=inner,
                                    stranded_resets=resets, rebuilds_kept=rebuilds_kept,
                                    rebuilds_tried=rebuilds_tried,
                                    burn_seconds=t_burn if burn < steps else time.perf_counter() - t0))


def hessian(post: Posterior, theta: np.ndarray, steps: np.ndarray) -> np.ndarray:
    """Hessian of log pi at each row of theta by central differences of
    adjoint gradients, steps[j] along parameter j; all 12 gradients of every
    row in one batched call. Symmetrised."""
    th = np.atleast_2d(theta)
    m, d = th.shape
    pts = np.repeat(th, 2 * d, axis=0)
    for j in range(d):
        pts[2 * j::2 * d, j] += steps[j]
        pts[2 * j + 1::2 * d, j] -= steps[j]
    _, g = post.loglik(pts, True)
    g = g.reshape(m, d, 2, d)
    H = (g[:, :, 0, :] - g[:, :, 1, :]) / (2 * steps[None, :, None])  # H[r, j, i] = d g_i / d theta_j
    return 0.5 * (H + H.transpose(0, 2, 1))


def _posdef_cov(H: np.ndarray, w: np.ndarray) -> np.ndarray:
    """Gaussian approximation of the posterior: covariance (|-H| + P)^{-1},
    with |.| the absolute eigenvalues of -H in width-scaled coordinates (a
    noisy or indefinite Hessian along a ridge stays positive) and P = 12 I
    the precision of a uniform distribution on the prior box (it bounds the
    variance along directions the likelihood does not constrain)."""
    A = -H * np.outer(w, w)
    ev, V = np.linalg.eigh(0.5 * (A + A.T))
    ev = np.abs(ev) + 12.0
    return (V / ev) @ V.T * np.outer(w, w)


def find_mode(post: Posterior, starts: np.ndarray, iters: int = 10, hess_rel: float = 1e-5):
    """Posterior mode from a few starting points by damped Newton steps:
    per iteration one batched adjoint call for the gradients and Hessians
    (central differences of gradients) of every start and one batched
    forward call that tries every damping level; a start keeps its best
    point. Returns (theta_map, log pi(theta_map), covariance (-H)^{-1} at the
    mode, history of the best log pi)."""
    w = post.prior.width
    th = np.array(np.atleast_2d(starts), dtype=np.float64)
    m, d = th.shape
    lp, _ = post.loglik(th, False)
    hist = [float(np.max(lp))]
    lams = np.array([0.0, 1e-3, 1e-2, 1e-1, 1.0, 10.0, 100.0])
    for _ in range(iters):
        ok = np.isfinite(lp)
        if not ok.any():
            break
        _, g = post.loglik(th, True)
        H = hessian(post, th, hess_rel * w)
        cands = []
        for r in range(m):
            A = -H[r] * np.outer(w, w)  # width-scaled coordinates
            gz = g[r] * w
            ev = np.abs(np.linalg.eigvalsh(0.5 * (A + A.T))).max() + 1e-300
            for lam in lams:
                try:
                    dz = np.linalg.solve(A + lam * ev * np.eye(d), gz)
                except np.linalg.LinAlgError:
                    dz = gz / ev
                cands.append(th[r] + dz * w)
        cands = np.array(cands)
        lc, _ = post.loglik(cands, False)
        lc = lc.reshape(m, len(lams))
        best = np.argmax(lc, axis=1)
        for r in range(m):
            if lc[r, best[r]] > lp[r]:
                th[r] = cands[r * len(lams) + best[r]]
                lp[r] = lc[r, best[r]]
        hist.append(float(np.max(lp)))
        if len(hist) > 2 and hist[-1] - hist[-2] < 1e-3:
            break
    r = int(np.argmax(lp))
    H = hessian(post, th[r], hess_rel * w)[0]
    cov = _posdef_cov(H, w)
    # second pass with steps of half a posterior standard deviation (at most
    # 1% of the prior width)
    sd = np.minimum(np.sqrt(np.diag(cov)), 0.02 * w)
    H = hessian(post, th[r], 0.5 * sd)[0]
    cov = _posdef_cov(H, w)
    return th[r].copy(), float(lp[r]), cov, hist


# Coordinates in which the Fisher-KPP scaling symmetry is an axis: the
# continuous model with this initial condition depends on (Dw / rho, rho T)
# only, so (Dw, rho, T) -> (c Dw, c rho, T / c) leaves the density unchanged
# and only the time discretisation and the prior box bound c. With
# u = (log Dw, log rho, x0, y0, z0, log T), the invariant coordinates are
# v = (log rho, log rho + log T, log Dw - log rho, x0, y0, z0): v_0 moves
# along the symmetry, v_1 and v_2 are its invariants.
INVARIANT_MAP = np.array([[0, 1, 0, 0, 0, 0],
                          [0, 1, 0, 0, 0, 1],
                          [1, -1, 0, 0, 0, 0],
                          [0, 0, 1, 0, 0, 0],
                          [0, 0, 0, 1, 0, 0],
                          [0, 0, 0, 0, 1, 0]], dtype=np.float64)


@dataclass
class LogPrior:
    """The prior of a LogCoords posterior, in its coordinates v = A u."""
    base: Prior
    log_idx: tuple
    A: np.ndarray

    def __post_init__(self):
        self.Ai = np.linalg.inv(self.A)

    def to_logu(self, v):
        return np.asarray(v, dtype=np.float64) @ self.Ai.T

    def to_theta(self, v):
        th = self.to_logu(v)
        with np.errstate(over="ignore"):  # far proposals map to inf, outside the prior
            th[..., list(self.log_idx)] = np.exp(th[..., list(self.log_idx)])
        return th

    def _ubox(self):
        lo, hi = self.base.lo.copy(), self.base.hi.copy()
        lo[list(self.log_idx)] = np.log(lo[list(self.log_idx)])
        hi[list(self.log_idx)] = np.log(hi[list(self.log_idx)])
        return lo, hi

    @property
    def width(self):
        """Extent of the prior box's image along each v coordinate."""
        lo, hi = self._ubox()
        return np.abs(self.A) @ (hi - lo)

    @property
    def lo(self):
        lo, hi = self._ubox()
        return np.minimum(self.A, 0) @ (hi - lo) + self.A @ lo

    @property
    def hi(self):
        return self.lo + self.width

    def _axis_line(self, v: np.ndarray, a: int):
        """The line v + t e_a through each row of v: the interval [t_lo, t_hi]
        of t inside the prior box (ok = non-empty) and the rate alpha of the
        prior density exp(alpha t) along it (every log coordinate is linear in
        t; alpha = sum over log coordinates of (A^{-1})_{i,a}). None when the
        line moves a non-log coordinate (the seed, whose prior is a voxel
        mask)."""
        col = self.Ai[:, a]
        logs = list(self.log_idx)
        if np.any(np.abs(np.delete(col, logs)) > 0):
            return None
        lo_u, hi_u = self._ubox()
        u = self.to_logu(v)
        t_lo = np.full(v.shape[0], -np.inf)
        t_hi = np.full(v.shape[0], np.inf)
        for i in logs:
            if col[i] == 0:
                continue
            b1 = (lo_u[i] - u[:, i]) / col[i]
            b2 = (hi_u[i] - u[:, i]) / col[i]
            t_lo = np.maximum(t_lo, np.minimum(b1, b2))
            t_hi = np.minimum(t_hi, np.maximum(b1, b2))
        ok = np.isfinite(t_lo) & np.isfinite(t_hi) & (t_hi > t_lo)
        return t_lo, t_hi, ok, float(col[logs].sum())

    def redraw_axis(self, v: np.ndarray, a: int, rng) -> np.ndarray:
        """Exact draw of coordinate a from the prior conditional given the
        others (rows of v): on the line v + t e_a the prior density is
        exp(alpha t) on [t_lo, t_hi] (_axis_line). Rows whose line moves a
        non-log coordinate, or misses the box, are returned unchanged."""
        v = np.array(np.atleast_2d(v), dtype=np.float64, copy=True)
        line = self._axis_line(v, a)
        if line is None:
            return v
        t_lo, t_hi, ok, alpha = line
        q = rng.random(v.shape[0])
        t = np.zeros(v.shape[0])
        if abs(alpha) < 1e-12:
            t[ok] = t_lo[ok] + q[ok] * (t_hi[ok] - t_lo[ok])
        else:
            # inverse CDF of exp(alpha t) on [t_lo, t_hi], in a stable form
            span = alpha * (t_hi[ok] - t_lo[ok])
            t[ok] = t_lo[ok] + np.log1p(q[ok] * np.expm1(span)) / alpha
        v[ok, a] += t[ok]
        return v

    def axis_log_marginal(self, v: np.ndarray, a: int) -> np.ndarray:
        """log of the prior density integrated over coordinate a through each
        row of v: the marginal prior of the other coordinates, the normaliser
        of redraw_axis's conditional (-inf where the line misses the prior's
        support)."""
        v = np.atleast_2d(np.asarray(v, dtype=np.float64))
        line = self._axis_line(v, a)
        if line is None:
            raise ValueError("coordinate a moves a non-log coordinate")
        t_lo, t_hi, ok, alpha = line
        out = np.full(v.shape[0], -np.inf)
        if not ok.any():
            return out
        mid = v[ok].copy()
        mid[:, a] += 0.5 * (t_lo[ok] + t_hi[ok])
        base = self.logp(mid)  # the seed-mask test, and the density at t = mid
        span = t_hi[ok] - t_lo[ok]
        if abs(alpha) < 1e-12:
            w = np.log(span)
        else:
            # integral of exp(alpha (t - mid)) over the interval
            w = np.log(2.0 * np.sinh(0.5 * alpha * span) / alpha)
        out[ok] = base + w
        return out

    def logp(self, v):
        """Uniform prior on theta as a density in v: the log-Jacobian sum of
        log theta_i over the log coordinates (the linear map's is a
        constant), -inf outside the box."""
        u = np.atleast_2d(self.to_logu(v))
        th = u.copy()
        th[:, list(self.log_idx)] = np.exp(th[:, list(self.log_idx)])
        return self.base.logp(th) + u[:, list(self.log_idx)].sum(axis=1)


@dataclass
class LogCoords:
    """A posterior in coordinates v = A u, u_i = log theta_i for i in
    log_idx (Dw, rho and T by default) and u_i = theta_i otherwise; A = I
    by default, INVARIANT_MAP for the scaling symmetry's coordinates. In u
    the curved Dw-rho-T ridge of the posterior is straight, in the invariant
    coordinates it is the v_0 axis. Densities include the Jacobian of the
    map; gradients are transformed with it."""
    post: object
    log_idx: tuple = (0, 1, 5)
    A: np.ndarray = None

    def __post_init__(self):
        if self.A is None:
            self.A = np.eye(len(self.post.prior.lo))
        self.A = np.asarray(self.A, dtype=np.float64)
        self.prior = LogPrior(self.post.prior, self.log_idx, self.A)

    def to_theta(self, v):
        return self.prior.to_theta(v)

    def to_u(self, th):
        u = np.array(th, dtype=np.float64, copy=True)
        u[..., list(self.log_idx)] = np.log(u[..., list(self.log_idx)])
        return u @ self.A.T

    @property
    def solves(self):
        return self.post.solves

    @property
    def seconds(self):
        return self.post.seconds

    def loglik(self, v, with_grad: bool):
        v = np.atleast_2d(v)
        u = self.prior.to_logu(v)
        th = self.to_theta(v)
        l, g = self.post.loglik(th, with_grad)
        jac = u[:, list(self.log_idx)].sum(axis=1)
        if with_grad:
            g = np.array(g, dtype=np.float64, copy=True)
            g[:, list(self.log_idx)] = g[:, list(self.log_idx)] * th[:, list(self.log_idx)] + 1.0
            g = g @ self.prior.Ai  # d/dv = A^{-T} d/du, row-wise
        return l + jac, g

    def surrogate(self, spost: "SurrogatePosterior") -> "SurrogatePosterior":
        """A theta-space surrogate posterior in the same coordinates."""
        return _LogSurrogate(spost, self)


class _LogSurrogate:
    def __init__(self, spost, lc):
        self.spost, self.lc = spost, lc

    def __getattr__(self, k):
        return getattr(self.spost, k)

    def logpost(self, v):
        v = np.atleast_2d(v)
        u = self.lc.prior.to_logu(v)
        return self.spost.logpost(self.lc.to_theta(v)) + u[:, list(self.lc.log_idx)].sum(axis=1)


def refine_cov(post, u_map: np.ndarray, cov: np.ndarray, span: float = 8.0, npts: int = 33,
               drop: float = 10.0, with_best: bool = False):
    """Gaussian approximation refined by profiles: log pi is evaluated along
    each eigenvector of the Laplace precision (in prior-width-scaled
    coordinates) at npts points out to +-span Laplace standard deviations,
    all directions in one batched call, and a parabola fitted to the points
    within `drop` of the centre gives that direction's standard deviation.
    Directions whose profile stays within `drop` over the whole span are
    rescanned 8x wider. A local Hessian misjudges directions along which log
    pi is kinked or nearly flat (the Dw-rho-T ridge); the profile fit sees
    the posterior's extent. Returns (covariance, per-direction sd ratio),
    and with with_best also the profile point of highest log pi and its
    value (above log pi(u_map) when u_map is short of the mode, e.g. part
    way along a narrow curved ridge)."""
    w = post.prior.width
    d = u_map.size
    A = np.linalg.inv(cov / np.outer(w, w))
    ev, V = np.linalg.eigh(0.5 * (A + A.T))
    sd = 1.0 / np.sqrt(ev)
    ts = np.linspace(-1.0, 1.0, npts)
    spans = np.full(d, span)
    ratio = np.ones(d)
    todo = list(range(d))
    best_u, best_lp = np.array(u_map, dtype=np.float64), -np.inf
    for _ in range(2):
        if not todo:
            break
        pts = np.concatenate([u_map + np.outer(ts * spans[k] * sd[k], V[:, k] * w) for k in todo])
        lp, _ = post.loglik(pts, False)
        fin = np.where(np.isfinite(lp), lp, -np.inf)
        if fin.max() > best_lp:
            best_lp = float(fin.max())
            best_u = pts[int(np.argmax(fin))].copy()
        lp = lp.reshape(len(todo), npts)
        again = []
        for j, k in enumerate(todo):
            x = ts * spans[k]
            dl = lp[j] - lp[j, npts // 2]
            sel = np.isfinite(dl) & (dl > -drop)
            if sel.all() and spans[k] == span:
                again.append(k)
                spans[k] *= 8.0
                continue
            if sel.sum() >= 3:
                c = np.polyfit(x[sel], dl[sel], 2)
                ratio[k] = np.sqrt(-0.5 / c[0]) if c[0] < 0 else spans[k]
            ratio[k] = min(max(ratio[k], 0.1), spans[k])
        todo = again
    sig = sd * ratio
    cov_r = (V * sig ** 2) @ V.T * np.outer(w, w)
    if with_best:
        return cov_r, ratio, best_u, best_lp
    return cov_r, ratio


def polish_mode(post, v_map: np.ndarray, lp_map: float, cov0: np.ndarray, polish: int = 8,
                iters: int = 5, gain: float = 1.0):
    """Mode search continued along the posterior's profiles: the posterior of
    the tumour model is a narrow curved ridge in (log rho T, log Dw/rho),
    along which damped Newton can stop short of the mode. While refine_cov's
    profiles hold a point more than `gain` nats above the current estimate,
    Newton restarts from that point (at most `polish` times). Returns
    (v_map, log pi(v_map), Laplace covariance, refined covariance, restarts)."""
    restarts = 0
    for _ in range(polish):
        cov, _, v_best, lp_best = refine_cov(post, v_map, cov0, with_best=True)
        if not lp_best > lp_map + gain:
            return v_map, lp_map, cov0, cov, restarts
        v_new, lp_new, cov_new, _ = find_mode(post, v_best[None], iters=iters)
        restarts += 1
        if lp_new > lp_map:
            v_map, lp_map, cov0 = v_new, lp_new, cov_new
    cov, _ = refine_cov(post, v_map, cov0)
    return v_map, lp_map, cov0, cov, restarts


def stable_dt0(n: int, L: float, dw_max: float, rho_max: float = 0.0) -> float:
    """Largest explicit step of the fixed time grid for diffusivities up to
    dw_max [cm^2/day] and growth rates up to rho_max [1/day]:
    dt = 0.99 h^2 / (6 Dw / L^2 + rho h^2 / 2), which keeps 12 a + b <= 1.98
    (a = dt Dw / (L h)^2, b = dt rho) so that the explicit step is stable
    where the density saturates too (rho_max = 0: the reference's diffusion
    rule alone)."""
    h = 1.0 / n
    return 0.99 * h * h / (6.0 * dw_max / (L * L) + 0.5 * rho_max * h * h)


def _base(post):
    return post.post if isinstance(post, LogCoords) else post


def _theta(post, u):
    return post.to_theta(u) if isinstance(post, LogCoords) else np.array(u, dtype=np.float64)


class AffineSurrogate:
    """Screening density for delayed acceptance around a reference point
    u_ref (normally the posterior mode): the final density is modelled as
      phi(u) = phi(u_ref) + J delta  [+ K_aa delta_a^2 / 2 + sum_i K_ai delta_a delta_i]
    with delta = u - u_ref, J from central differences of the batched
    solver's densities (steps[p] along coordinate p) and, with quad_axis = a,
    the second-order terms along coordinate a (the scaling symmetry's axis in
    the invariant coordinates, along which the posterior ridge curves) from
    the same central differences and 4 mixed-difference solves per other
    coordinate; all solves of a build go through one batched call. log L of
    the field comes from the library's affine model and likelihood kernel
    (gbg_affine_loglik), whose basis fields are J and the K columns. A
    handle holds one affine model: the latest build on it is the active one."""

    def __init__(self, post, u_ref: np.ndarray, steps: np.ndarray, quad_axis=None):
        self.post, self.base = post, _base(post)
        self.prior = post.prior
        self.quad_axis = quad_axis
        self.evals = 0
        self.calls = 0
        self.seconds = 0.0
        self.rebuild(u_ref, steps)
        h = self.base.handle
        self.gpu_chain_ready = hasattr(h, "affine_chain")
        if self.gpu_chain_ready:
            base_prior = self.prior.base if isinstance(self.prior, LogPrior) else self.prior
            h.affine_set_prior_mask(base_prior.seed_mask)

    def chain(self, v: np.ndarray, steps: int, step: float, chol: np.ndarray, axis, axis_prob: float,
              seed: int, ind=None):
        """The inner chain of da on the GPU (gbg_affine_chain): `steps` steps
        for every row of v on this screen's posterior, the same moves as
        inner_chain (random walk step * chol xi on the coordinates other than
        `axis`, with probability axis_prob a redraw of `axis` from its prior
        conditional, with ind = (probability, mean, factor) independence
        proposals). Returns (end points, log pi* at the start points, log pi*
        at the end points, random-walk acceptance fraction); the independence
        moves' acceptance is kept in last_ind_accept."""
        pr = self.prior
        if isinstance(pr, LogPrior):
            Ai, log_mask, lo, hi = pr.Ai, sum(1 << i for i in pr.log_idx), pr.base.lo, pr.base.hi
        else:
            Ai, log_mask, lo, hi = np.eye(6), 0, pr.lo, pr.hi
        ip, im, ig = (0.0, None, None) if ind is None else ind
        t0 = time.perf_counter()
        y, l0, l1, cnt = self.base.handle.affine_chain(
            v, steps, seed, step=step, chol=chol, axis=-1 if axis is None else axis,
            axis_prob=axis_prob if axis is not None else 0.0, u_ref=self.u_ref,
            quad_axis=-1 if self.quad_axis is None else self.quad_axis, Ai=Ai, log_mask=log_mask,
            lo=lo, hi=hi, ind_prob=ip, ind_mean=im, ind_chol=ig)
        self.seconds += time.perf_counter() - t0
        self.calls += 1
        self.evals += int(np.atleast_2d(v).shape[0]) * (steps + 1)
        self.last_ind_accept = float(cnt[:, 4].sum() / cnt[:, 5].sum()) if cnt[:, 5].sum() else 0.0
        rw = cnt[:, 1].sum()
        return y, l0, l1, float(cnt[:, 0].sum() / rw) if rw else 0.0

    def _coeffs(self, delta: np.ndarray) -> np.ndarray:
        if self.quad_axis is None:
            return delta
        a = self.quad_axis
        others = [i for i in range(delta.shape[1]) if i != a]
        return np.concatenate([delta, 0.5 * delta[:, a:a + 1] ** 2,
                               delta[:, a:a + 1] * delta[:, others]], axis=1)

    def rebuild(self, u_ref: np.ndarray, steps: np.ndarray):
        """Re-build at u_ref with finite-difference steps `steps`."""
        post, base = self.post, self.base
        self.u_ref = np.array(u_ref, dtype=np.float64)
        d = self.u_ref.size
        steps = np.asarray(steps, dtype=np.float64)
        pts = np.repeat(self.u_ref[None], 2 * d + 1, axis=0)
        for p in range(d):
            pts[1 + 2 * p, p] += steps[p]
            pts[2 + 2 * p, p] -= steps[p]
        a = self.quad_axis
        others = [] if a is None else [i for i in range(d) if i != a]
        mixed = []
        for i in others:
            for sa, si in ((1, 1), (1, -1), (-1, 1), (-1, -1)):
                q = self.u_ref.copy()
                q[a] += sa * steps[a]
                q[i] += si * steps[i]
                mixed.append(q)
        if mixed:
            pts = np.concatenate([pts, np.array(mixed)])
        th = _theta(post, pts)
        h = base.handle
        cap = max(1, h.max_samples)
        phis = []
        for s0 in range(0, len(th), cap):
            r = h.batch_solve([tuple(x) for x in th[s0:s0 + cap]], base.L, ic_peak=base.ic_peak,
                              ic_sigma=base.ic_sigma, with_loglik=False, want_phi=True, dt0=base.dt0)
            phis.append(r["phi"].reshape(r["phi"].shape[0], -1))
        phis = np.concatenate(phis).astype(np.float64)
        self.phi0 = phis[0].astype(np.float32)
        basis = [(phis[1 + 2 * p] - phis[2 + 2 * p]) / (2 * steps[p]) for p in range(d)]
        if a is not None:
            basis.append((phis[1 + 2 * a] + phis[2 + 2 * a] - 2 * phis[0]) / steps[a] ** 2)
            for j, i in enumerate(others):
                f = phis[2 * d + 1 + 4 * j: 2 * d + 5 + 4 * j]
                basis.append((f[0] - f[1] - f[2] + f[3]) / (4 * steps[a] * steps[i]))
        self.J = np.stack(basis)
        h.affine_set(self.phi0, self.J.astype(np.float32))

    def state(self):
        """The current build (for restore)."""
        return (self.u_ref.copy(), self.phi0.copy(), self.J.copy())

    def restore(self, state):
        """Make an earlier build the active one again."""
        self.u_ref, self.phi0, self.J = (np.array(x) for x in state)
        self.base.handle.affine_set(self.phi0, self.J.astype(np.float32))

    def logpost(self, u: np.ndarray) -> np.ndarray:
        u = np.atleast_2d(u)
        lp = self.prior.logp(u)
        out = np.full(u.shape[0], -np.inf)
        ok = np.isfinite(lp)
        if ok.any():
            t0 = time.perf_counter()
            out[ok] = self.base.handle.affine_loglik(self._coeffs(u[ok] - self.u_ref))
            self.seconds += time.perf_counter() - t0
            self.calls += 1
            self.evals += int(ok.sum())
        return out + lp


@dataclass
class PipelineResult:
    result: ChainResult      # the DA chains (sampler coordinates)
    theta: np.ndarray        # post-burn-in draws in theta, (steps, chains, 6)
    v_map: np.ndarray
    cov: np.ndarray
    setup_seconds: float     # prior screen + mode + profiles + surrogate
    sample_seconds: float    # the post-burn-in generations
    burn_seconds: float
    surrogate: object = None   # the stage-1 surrogate as adapted in burn-in
    solver_seconds: float = 0.0     # inside the batched solver calls (whole DA run)
    surrogate_seconds: float = 0.0  # inside the surrogate calls (whole DA run)


def sample_posterior(handle, L: float, prior: Prior, dt0: float, rng, chains: int = 64,
                     generations: int = 300, burn: int = 100, inner: int = 16,
                     screen: int = 512, screen_draws=None, ic_peak: float = 0.1,
                     ic_sigma: float = 1.0, adapt_pool: bool = True, adapt: bool = True,
                     rebuild_every: int = 25, reset_stranded: bool = True,
                     polish: int = 8, ind_prob: float = 0.0) -> PipelineResult:
    """The batched + adjoint + surrogate posterior sampler (dt0 < 0, the
    scaled time grid, makes the likelihood invariant along the scaling
    symmetry, whose coordinate is then drawn exactly from its prior
    conditional; dt0 > 0 works too, with that move an ordinary MH step):
      1. log pi of `screen` prior draws in batched solves; the best four start
      2. damped Newton with batched adjoint gradients and Hessians (find_mode)
         in the scaling symmetry's coordinates (INVARIANT_MAP)
      3. the Laplace covariance refined by batched profiles (refine_cov);
         while a profile point lies more than 1 nat above the mode estimate,
         Newton restarts from it (at most `polish` times)
      4. delayed acceptance with the affine (tangent) surrogate around the
         mode, `chains` chains started from the refined Gaussian, proposal
         covariance and surrogate adapted to the population during burn-in
         and frozen after it.
    screen_draws: theta rows to screen instead of drawing from the prior
    (the caller's prior sampler)."""
    post = LogCoords(Posterior(handle, L, dt0, prior, ic_peak=ic_peak, ic_sigma=ic_sigma),
                     A=INVARIANT_MAP)
    t0 = time.perf_counter()
    if screen_draws is None:
        raise ValueError("screen_draws: theta rows drawn from the prior")
    dv = post.to_u(np.asarray(screen_draws, dtype=np.float64))
    ld, _ = post.loglik(dv, False)
    starts = dv[np.argsort(ld)[::-1][:4]]
    v_map, lp_map, cov0, _ = find_mode(post, starts, iters=10)
    v_map, lp_map, cov0, cov, _ = polish_mode(post, v_map, lp_map, cov0, polish=polish)
    sd = np.sqrt(np.diag(cov))
    Lc = np.linalg.cholesky(cov)
    sur = AffineSurrogate(post, v_map, 0.5 * sd, quad_axis=0)
    setup = time.perf_counter() - t0
    # starting points from the refined Gaussian, the symmetry axis redrawn
    # from its prior conditional, redrawn until inside the prior
    def draw(k):
        v = v_map + rng.standard_normal((k, v_map.size)) @ Lc.T
        return post.prior.redraw_axis(v, 0, rng)
    v0 = draw(chains)
    for _ in range(100):
        bad = ~np.isfinite(post.prior.logp(v0))
        if not bad.any():
            break
        v0[bad] = draw(int(bad.sum()))
    v0[~np.isfinite(post.prior.logp(v0))] = v_map
    run = Posterior(handle, L, dt0, prior, ic_peak=ic_peak, ic_sigma=ic_sigma)
    r = da(LogCoords(run, A=INVARIANT_MAP), sur, v0, generations, 2.38 / np.sqrt(v_map.size), rng,
           inner=inner, burn=burn, chol=Lc, adapt=adapt, rebuild_every=rebuild_every, axis=0,
           adapt_pool=adapt_pool, reset_stranded=reset_stranded, ind_prob=ind_prob)
    burn_s = r.history["burn_seconds"]
    return PipelineResult(r, post.to_theta(r.samples[burn:]), v_map, cov, setup, r.seconds - burn_s,
                          burn_s, surrogate=sur, solver_seconds=run.seconds,
                          surrogate_seconds=sur.seconds)


@dataclass
class TmcmcResult:
    theta: np.ndarray        # final population (N, d), posterior draws
    loglik: np.ndarray       # their log L (N,)
    p: list                  # tempering exponents, 0 = p_0 < ... < p_m = 1
    log_evidence: float      # log of the estimated marginal likelihood
    accept: list             # Metropolis acceptance per stage
    solves: int
    seconds: float


def _tempering_step(ll: np.ndarray, room: float, cov_tol: float) -> float:
    """The increment q in (0, room] of the tempering exponent whose weights
    exp(q (ll - max ll)) have coefficient of variation cov_tol (room when
    even q = room stays below it); bisection, the CoV growing with q."""
    d = ll - ll.max()

    def cov(q):
        w = np.exp(q * d)
        return w.std() / w.mean()

    if cov(room) <= cov_tol:
        return room
    lo, hi = 0.0, room
    for _ in range(100):
        mid = 0.5 * (lo + hi)
        if cov(mid) > cov_tol:
            hi = mid
        else:
            lo = mid
        if hi - lo <= 1e-12 * room:
            break
    return max(lo, 1e-12 * room)


def tmcmc(post, theta0: np.ndarray, rng, cov_tol: float = 1.0, beta2: float = 0.04,
          max_chain: int = 1, max_stages: int = 200, steps_per_state: int = 3,
          target_accept: float = 0.3) -> TmcmcResult:
    """Transitional MCMC (Ching & Chen 2007; the sampler the reference's
    workflow runs outside its code: one brain + likelihood process pair per
    sample) on the batched solver. theta0: N draws from the prior (rows, in
    post's coordinates); post.loglik gives log L + log prior and
    post.prior.logp the log prior. Stage j targets prior * L^p_j:
      1. the increment of p is the one whose plausibility weights
         w_i = L_i^(p_j+1 - p_j) have coefficient of variation cov_tol;
         log S_j = log mean(w) adds to the log evidence;
      2. proposal covariance beta2 * the weighted covariance of the
         population;
      3. N leaders are drawn with probabilities w / sum(w); a leader drawn c
         times starts a Metropolis chain whose c states are population
         members (max_chain > 0 splits it into chains of at most max_chain
         states, each from the leader);
      4. all chains step in lock-step: every step is one batched solve of
         the active chains' proposals; a chain records its state after every
         `steps_per_state` steps (1: Ching & Chen's chains).
    With target_accept, beta2 is rescaled after every stage by
    exp(2 (acceptance - target_accept)) (the proposal scale adaptation of
    Betz, Papaioannou & Straub 2016). max_chain = 0, steps_per_state = 1,
    target_accept = None is Ching & Chen's original. The defaults (every
    resampled state its own chain of 3 steps, adapted scale) keep all N
    chains in every batched solve, and they remove the bias of the
    original's log evidence: chains of correlated states from one leader make
    the next stage's weights and tempering step depend on few distinct points
    (on a 1-D Gaussian inside a box the original is low by 0.04 +- 0.006 at
    N = 2000, single-state chains within 0.01). Ends when p reaches 1 (or
    after max_stages)."""
    th = np.array(np.atleast_2d(theta0), dtype=np.float64)
    N, d = th.shape
    t0 = time.perf_counter()
    solves0 = getattr(post, "solves", 0)
    lpost, _ = post.loglik(th, False)
    lpr = post.prior.logp(th)
    ll = np.where(np.isfinite(lpr), lpost - lpr, -np.inf)
    if not np.isfinite(ll).any():
        raise ValueError("no prior draw has a finite likelihood")
    p = 0.0
    ps, acc, log_ev = [0.0], [], 0.0
    for _ in range(max_stages):
        if p >= 1.0:
            break
        fin = np.isfinite(ll)
        q = _tempering_step(ll[fin], 1.0 - p, cov_tol)
        if p + q >= 1.0 - 1e-12:
            q = 1.0 - p
        llmax = ll[fin].max()
        w = np.where(fin, np.exp(q * (ll - llmax)), 0.0)
        log_ev += np.log(w.sum() / N) + q * llmax
        wn = w / w.sum()
        p += q
        mu = wn @ th
        dev = th - mu
        cov = beta2 * (dev * wn[:, None]).T @ dev
        Lc = np.linalg.cholesky(cov + 1e-12 * np.diag(np.diag(cov)) + 1e-300 * np.eye(d))
        counts = rng.multinomial(N, wn)
        starts, lens = [], []
        for i in np.flatnonzero(counts):
            c = int(counts[i])
            while c > 0:
                k = c if max_chain <= 0 else min(c, max_chain)
                starts.append(i)
                lens.append(k)
                c -= k
        lens = np.array(lens)
        cur = th[starts].copy()
        cur_ll = ll[starts].copy()
        cur_lpr = lpr[starts].copy()
        new_th, new_ll, new_lpr = [], [], []
        n_acc = n_try = 0
        for k in range(int(lens.max()) * steps_per_state):
            act = np.flatnonzero(lens > k // steps_per_state)
            prop = cur[act] + rng.standard_normal((act.size, d)) @ Lc.T
            pl = post.prior.logp(prop)
            ok = np.isfinite(pl)
            pll = np.full(act.size, -np.inf)
            if ok.any():
                lq, _ = post.loglik(prop[ok], False)
                pll[ok] = lq - pl[ok]
            with np.errstate(invalid="ignore"):
                logr = (pl + p * pll) - (cur_lpr[act] + p * cur_ll[act])
            a = ok & np.isfinite(pll) & (np.log(rng.random(act.size)) < logr)
            sel = act[a]
            cur[sel], cur_ll[sel], cur_lpr[sel] = prop[a], pll[a], pl[a]
            n_acc += int(a.sum())
            n_try += act.size
            if (k + 1) % steps_per_state == 0:
                new_th.append(cur[act].copy())
                new_ll.append(cur_ll[act].copy())
                new_lpr.append(cur_lpr[act].copy())
        th = np.concatenate(new_th)
        ll = np.concatenate(new_ll)
        lpr = np.concatenate(new_lpr)
        ps.append(p)
        acc.append(n_acc / max(n_try, 1))
        if target_accept is not None:
            beta2 *= np.exp(2.0 * (acc[-1] - target_accept))
    return TmcmcResult(th, ll, ps, float(log_ev), acc, getattr(post, "solves", 0) - solves0,
                       time.perf_counter() - t0)


def propagate(handle, L: float, theta: np.ndarray, dt0: float = 0.0, ic_peak: float = 0.1,
              ic_sigma: float = 1.0, reference_rules: bool = False):
    """Posterior propagation: the per-cell mean and variance of the final
    densities of the samples theta (rows), in one batched solve + statistics
    call (gbg_batch_statistics; the reference's propagation tool over the
    samples' HGG_data.dat files, Glioma_HG_Propagation.cpp:346-440).
    len(theta) <= the handle's max_samples. reference_rules keeps the tool's
    zero planes at index 0."""
    th = np.atleast_2d(np.asarray(theta, dtype=np.float64))
    if th.shape[0] > handle.max_samples:
        raise ValueError("more samples than the handle's max_samples")
    return handle.batch_statistics([tuple(x) for x in th], L, ic_peak=ic_peak, ic_sigma=ic_sigma,
                                   dt0=dt0, reference_rules=reference_rules)


def rhat(samples: np.ndarray) -> np.ndarray:
    """Split-R-hat per parameter of (steps, chains, d) draws (Gelman-Rubin
    on the chains cut in halves): near 1 when the chains agree, well above
    1 while they still sample different regions."""
    n = samples.shape[0] // 2
    x = np.concatenate([samples[:n], samples[n:2 * n]], axis=1)
    w = x.var(axis=0, ddof=1).mean(axis=0)
    b = n * x.mean(axis=0).var(axis=0, ddof=1)
    var_plus = (n - 1) / n * w + b / n
    return np.sqrt(var_plus / np.maximum(w, 1e-300))


def _autocov(x: np.ndarray) -> np.ndarray:
    n = x.size
    f = np.fft.rfft(x - x.mean(), n=2 * n)
    ac = np.fft.irfft(f * np.conjugate(f))[:n]
    return ac / n


def ess(samples: np.ndarray, within: bool = False) -> np.ndarray:
    """Effective sample size per parameter of (steps, chains, d) draws:
    chain-averaged autocorrelation (split-free version of the multi-chain
    estimator) with Geyer's initial monotone sequence truncation. With
    within=True only the chains' own autocorrelation counts (the pooled
    within-chain autocorrelation, rho_t = mean acov_t / mean acov_0): a
    conservative figure that gives no credit for the spread of the chains'
    starting points."""
    n, m, d = samples.shape
    out = np.zeros(d)
    for j in range(d):
        x = samples[:, :, j]
        acov = np.stack([_autocov(x[:, c]) for c in range(m)])
        w = acov[:, 0].mean() * n / max(n - 1, 1)
        b = n * x.mean(axis=0).var(ddof=1) if m > 1 else 0.0
        var_plus = (n - 1) / n * w + b / n
        if within:
            var_plus = acov[:, 0].mean()
        if var_plus <= 0:
            out[j] = float(n * m)
            continue
        rho = 1.0 - (w - acov.mean(axis=0)) / var_plus
        if within:
            rho = acov.mean(axis=0) / var_plus
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
