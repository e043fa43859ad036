"""Benchmark: forward solves per second at 128^3 for a batched population.

Workload (one "step"): a population of S = 512 independent forward solves of
the Fisher-Kolmogorov tumour-growth model on a uniform 128^3 grid sharing one
synthetic anatomy, each with its own (Dw, rho, seed position, T) drawn from
the uniform priors, each integrated with the reference's explicit-Euler time
loop (13..760 steps), followed by each sample's imaging log-likelihood against
synthetic PET/T1/T2 observations of a hidden ground truth. FP32 state,
log-likelihood accumulated in FP64.

  value  : solves/s with the sample parameters already resident on the GPU
           (gbg_batch_solve_device), CUDA events on the library's stream
  e2e    : solves/s through the host C-ABI entry gbg_batch_solve (parameters
           copied in, one CUDA graph launch, log-likelihoods and step counts
           copied out each step)
  roofline: the population kernel's algorithmic bytes (8 B per cell-step it
           computes, plus 8/S B of shared anatomy) over its event-timed
           duration, against the measured HBM copy bandwidth; the skipping
           kernel computes only cells whose value can be nonzero, and the
           dense-equivalent figure (every cell of every step) is given beside
  cpu_baseline: the oracle's block-lab restatement of the reference's CPU
           step (FP32, all host cores) on a bounded sample, scaled to solves/s

`--impl reference` times that CPU restatement alone as the reference arm.
Multi-GPU (torchrun): every rank solves its own population (weak scaling, no
collective on the data path); timing is the max over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N = 128
S = 512
LIK = (0.0025, 1.0, 0.7, 0.25, 0.09)
METRIC = "forward solves/s at 128^3 (batched population of 512, with log-likelihood)"


def set_population(samples):
    global S
    S = samples


def rank_info():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("LOCAL_RANK", "0")),
            int(os.environ.get("WORLD_SIZE", "1")))


def max_over_ranks(value: float, world: int, device) -> float:
    """The largest of every rank's value (the job's time is its slowest
    rank's); a no-op on one rank."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([value], dtype=torch.float64, device=device)
    if world > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(samples_per_rank: int, world: int, seconds_per_step: float) -> float:
    """Whole-job solves/s: every rank solves its own population (weak scaling,
    no collective on the data path), the step lasts as long as the slowest."""
    return world * samples_per_rank / seconds_per_step


def make_workload(seed_offset=0):
    from gliomauq_gb300 import synthetic as Syn
    an = Syn.make_anatomy(N, seed=0)
    prior = Syn.draw_prior(an, S, seed=1 + seed_offset)
    truth = Syn.draw_prior(an, 1, seed=10_000)[0]
    return an, prior, truth


def mean_cell_steps(an, prior):
    from gliomauq_gb300 import synthetic as Syn
    steps = [Syn.num_steps(Syn.reference_dt(N, p.Dw, an.L)[0], p.T) for p in prior]
    return float(np.mean(steps)) * N ** 3, steps


def observations(h, an, truth):
    """Synthetic observations of the hidden truth, solved on the GPU."""
    from gliomauq_gb300 import synthetic as Syn
    res = h.batch_solve([truth.as_tuple()], an.L, with_loglik=False, want_phi=True)
    u = res["phi"][0].astype(np.float64)
    return Syn.make_observations(u, an, seed=3, centre_xyz=(truth.x0, truth.y0, truth.z0),
                                 radius_vox=27.0)


def measured_peaks():
    for p in (os.path.join(ROOT, "MEASURED_PEAKS.json"),):
        if os.path.exists(p):
            with open(p) as f:
                d = json.load(f)
            return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class Clocks:
    """nvidia-smi clock sampling during the timed region."""

    def __init__(self, gpu_index):
        self.path = tempfile.mktemp(suffix=".csv")
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.f = open(self.path, "w")
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(gpu_index), f"--query-gpu={q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        self.f.close()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for name, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(sm)}


# The block-lab port against the reference's own TBB pipeline (compiled in place
# with _MRAG_TBB_NTHREADS_HINT = cores on a project-written thread-backed TBB
# stand-in; oracle/Makefile target ref_harness_f32_tbb), same 128^3 bench sample
# and steps, on the 8-core x86 build machine: port / reference cell-steps/s.
PORT_OVER_REFERENCE = {"threads_1": 10.285e6 / 10.229e6, "threads_8": 77.37e6 / 56.28e6}


def cpu_baseline(an, prior, seconds=12.0, obs=None):
    """The oracle's block-lab restatement of the reference CPU step, all cores,
    on one sample of the workload for about `seconds`, plus the reference's
    likelihood (HGG_Likelihood restated) on the final field when `obs` is
    given; extrapolated to solves/s with the population's mean step count."""
    from gliomauq_gb300 import synthetic as Syn
    from oracle import oracle
    p = prior[0]
    dt, dw, dg = Syn.reference_dt(N, p.Dw, an.L, f32=True)
    phi0 = Syn.gaussian_ic(an, p.x0, p.y0, p.z0)
    g = oracle.BlockGrid(an.p_w, an.p_g, phi0)
    cores = os.cpu_count() or 1
    g.steps(dw, dg, p.rho, dt, 1, cores)  # warm-up
    steps, t0 = 0, time.perf_counter()
    while True:
        g.steps(dw, dg, p.rho, dt, 4, cores)
        steps += 4
        el = time.perf_counter() - t0
        if el >= seconds:
            break
    cs = steps * N ** 3 / el
    per_solve, _ = mean_cell_steps(an, prior)
    lik_s = 0.0
    if obs is not None:
        u = g.phi().astype(np.float64)
        t1 = time.perf_counter()
        oracle.loglik(u, obs.pet, obs.t1, obs.t2, obs.points, LIK, 3, 2, True)
        lik_s = time.perf_counter() - t1
    solve_s = per_solve / cs + lik_s
    return dict(value=1.0 / solve_s, unit="solves/s", cores=cores, kind="port",
                extrapolated=True, measured_cell_steps=steps * N ** 3, measured_seconds=el,
                mean_cell_steps_per_solve=per_solve, loglik_seconds_per_solve=lik_s,
                port_over_reference_x86=PORT_OVER_REFERENCE,
                sample=f"{steps} steps of one 128^3 sample ({el:.1f} s) through the block-lab "
                       f"restatement of the reference CPU step (FP32 Real, {cores} threads): "
                       f"{cs / 1e6:.1f} Mcell-steps/s, extrapolated to the population's mean "
                       f"{per_solve / N ** 3:.1f} steps per solve"
                       + (f", plus the likelihood ({1e3 * lik_s:.1f} ms per solve)" if obs is not None
                          else ""))


def mcmc_comparison(device, n=128, chains=64, generations=300, burn=100, inner=64,
                    plain_chains=4, plain_steps=1500, plain_burn=300, ref_generations=500,
                    plain_cap_s=150.0, unet=True, mala_steps=0, mala_burn=100, ind_prob=0.0,
                    unet_train=20000, unet_epochs=3, seed=0):
    """Posterior effective samples per second at n^3 on one synthetic
    patient, plain single-solve MCMC against the batched + adjoint +
    surrogate pipeline, both in the scaling symmetry's coordinates
    (log rho, log rho T, log Dw/rho, x0, y0, z0) with the same Laplace
    preconditioning:
      * plain (gliomauq_gb300.mcmc.plain_chains): `plain_chains` chains run
        one after another, one forward solve per step; random walk on the
        identified coordinates with the pipeline's refined Laplace
        covariance, the symmetry axis redrawn from its prior conditional
        every step; more steps are added until split R-hat <= 1.05 and the
        theta means' Monte Carlo errors are within 0.5 % (at most
        `plain_cap_s` seconds);
      * pipeline (gliomauq_gb300.mcmc.sample_posterior): batched prior
        screen, adjoint Newton mode and Hessian, profile-refined Gaussian,
        then delayed acceptance with the affine tangent surrogate over
        `chains` lock-step chains.
    Both target the same posterior (scaled time grid); the observations come
    from the same model. The setup (screen, mode, covariance) is shared and
    reported separately; ESS/s counts the post-burn-in sampling time of
    each. A second, longer pipeline run from fresh chains gives the
    reference posterior mean that both samplers' means are checked against
    (2 % per theta coordinate). The learned U-Net surrogate is measured as a
    stage-1 screen in the same delayed-acceptance sampler. With mala_steps,
    the adjoint MALA configuration too: 64 chains of preconditioned MALA
    (adjoint gradients, checkpoints every 50 steps), step size adapted to
    0.574 acceptance during mala_burn steps. The population kernel is the
    autotuner's choice for both samplers."""
    from gliomauq_gb300 import _lib, mcmc, synthetic as Syn
    an = Syn.make_anatomy(n, seed=0)
    truth = Syn.draw_prior(an, 1, seed=10_000)[0]
    rng = np.random.default_rng(seed)
    h = _lib.Handle(n, "f32", device=device, max_samples=512)
    h.set_anatomy(an.p_w, an.p_g)
    tune_cache = os.path.join(ROOT, "gliomauq_gb300", "_build", "tune.json")
    os.makedirs(os.path.dirname(tune_cache), exist_ok=True)
    variant = h.autotune(probe_samples=64, cache_path=tune_cache)
    prior = mcmc.Prior.from_anatomy(an)
    # scaled time grid: the reference's step rule with the reaction's share of
    # the stability bound, per sample, with a shortened last step (smooth in
    # tend, Dw and rho, stable where the density saturates, and it keeps the
    # scaling symmetry)
    dt0 = -1.0
    # observations from the same forward model the samplers use
    u = h.batch_solve([truth.as_tuple()], an.L, with_loglik=False, want_phi=True,
                      dt0=dt0)["phi"][0]
    obs = Syn.make_observations(u.astype(np.float64), an, seed=3,
                                centre_xyz=(truth.x0, truth.y0, truth.z0),
                                radius_vox=27.0 * n / 128)
    h.set_observations(obs.pet, obs.t1, obs.t2, obs.points, LIK, step_pet=3, step_ti=2)
    screen = np.array([p.as_tuple() for p in Syn.draw_prior(an, 512, seed=99)])
    res = mcmc.sample_posterior(h, an.L, prior, dt0, rng, chains=chains, generations=generations,
                                burn=burn, inner=inner, screen_draws=screen, ind_prob=ind_prob)
    lc = mcmc.LogCoords(mcmc.Posterior(h, an.L, dt0, prior), A=mcmc.INVARIANT_MAP)
    names = ["log c (symmetry axis)", "log rho T", "log Dw/rho", "x0", "y0", "z0"]

    def diagnostics(theta, seconds):
        v = lc.to_u(theta)  # sampler-independent invariant coordinates
        e, ew, rh = mcmc.ess(v), mcmc.ess(v, within=True), mcmc.rhat(v)
        ident = slice(1, 6)
        return {"ess": e.tolist(), "ess_within": ew.tolist(), "rhat": rh.tolist(),
                "seconds": seconds,
                "ess_per_s_identified": float(e[ident].min() / seconds),
                "ess_per_s_symmetry_axis": float(e[0] / seconds),
                "ess_per_s_all": float(e.min() / seconds),
                "mean_theta": theta.reshape(-1, 6).mean(axis=0).tolist(),
                "mean_v": v.reshape(-1, 6).mean(axis=0).tolist(),
                "sd_v": v.reshape(-1, 6).std(axis=0).tolist()}

    def start_points(k, scale=2.0):
        """Dispersed starts: the refined Gaussian widened by `scale`, the
        symmetry axis from its prior conditional, inside the prior."""
        Lc = np.linalg.cholesky(res.cov)
        v = np.empty((0, 6))
        while len(v) < k:
            d = res.v_map + scale * rng.standard_normal((4 * k, 6)) @ Lc.T
            d = lc.prior.redraw_axis(d, 0, rng)
            v = np.concatenate([v, d[np.isfinite(lc.prior.logp(d))]])
        return v[:k]

    th = res.theta
    d_pipe = diagnostics(th, res.sample_seconds)
    half = chains // 2
    va = lc.to_u(th[:, :half]).reshape(-1, 6).mean(axis=0)
    vb = lc.to_u(th[:, half:]).reshape(-1, 6).mean(axis=0)
    d_pipe["halves_mean_diff_in_sd"] = (np.abs(va - vb) / np.array(d_pipe["sd_v"])).tolist()

    # plain single-solve chains, same coordinates and preconditioning
    post1 = mcmc.Posterior(h, an.L, dt0, prior)
    lc1 = mcmc.LogCoords(post1, A=mcmc.INVARIANT_MAP)
    r1 = mcmc.plain_chains(lc1, start_points(plain_chains), plain_burn + plain_steps, res.cov, rng,
                           burn=plain_burn)
    draws = r1.samples[plain_burn:]
    t_plain = r1.seconds - r1.history["burn_seconds"]
    acc_n, acc_sum = plain_steps * plain_chains, r1.accept * plain_steps * plain_chains
    t_round = r1.seconds
    spent = r1.seconds

    def converged(v):
        """split R-hat <= 1.05 and every theta mean's Monte Carlo standard
        error (posterior sd / sqrt(ESS)) within 0.5 % of the mean, a quarter
        of the 2 % the means are checked to"""
        th_v = lc.to_theta(v)
        mcse = th_v.reshape(-1, 6).std(axis=0) / np.sqrt(mcmc.ess(th_v))
        return (np.max(mcmc.rhat(v)) <= 1.05 and
                np.all(mcse <= 0.005 * np.abs(th_v.reshape(-1, 6).mean(axis=0))))

    while not converged(draws) and spent + t_round < plain_cap_s:
        more = mcmc.plain_chains(lc1, draws[-1], plain_steps, res.cov, rng, burn=0, step=r1.step)
        draws = np.concatenate([draws, more.samples])
        t_plain += more.seconds
        spent += more.seconds
        t_round = more.seconds
        acc_n += plain_steps * plain_chains
        acc_sum += more.accept * plain_steps * plain_chains
    th_plain = lc.to_theta(draws)
    d_plain = diagnostics(th_plain, t_plain)
    # reference posterior mean: a longer pipeline run from fresh chains with
    # the same setup (its surrogate as adapted above; stage 2 keeps it exact)
    post_r = mcmc.LogCoords(mcmc.Posterior(h, an.L, dt0, prior), A=mcmc.INVARIANT_MAP)
    rr = mcmc.da(post_r, res.surrogate, start_points(chains, 1.0), ref_generations + burn,
                 2.38 / np.sqrt(6), np.random.default_rng(12345), inner=inner, burn=burn,
                 chol=np.linalg.cholesky(res.cov), adapt=True, axis=0, ind_prob=ind_prob)
    th_ref = lc.to_theta(rr.samples[burn:]).reshape(-1, 6)
    ref_mean = th_ref.mean(axis=0)
    ref_sd = th_ref.std(axis=0)

    def mean_check(theta):
        m = theta.reshape(-1, 6).mean(axis=0)
        rel = np.abs(m - ref_mean) / np.abs(ref_mean)
        return {"rel_err": rel.tolist(), "err_in_sd": (np.abs(m - ref_mean) / ref_sd).tolist(),
                "within_2pct": bool(np.all(rel <= 0.02))}

    out = {
        "grid": n, "time_grid": "scaled, stable: dt = 0.99 h^2 / (6 Dw / L^2 + rho h^2 / 2) per "
                                "sample, last step shortened to end at T", "coordinates": names,
        "posterior": "synthetic truth, PET/T1/T2 likelihood, scaled-time-grid model (data and "
                     "inference)",
        "truth": list(truth.as_tuple()),
        "note": "the model depends on (Dw/rho, rho T) only (the scaled grid keeps this "
                "symmetry of the continuous model): along (c Dw, c rho, T/c) the posterior is the "
                "prior's, and both samplers draw that coordinate exactly from its prior "
                "conditional; ESS/s is reported for the identified coordinates and for the "
                "symmetry axis separately",
        "setup_seconds": res.setup_seconds,
        "plain": dict(sampler=f"{plain_chains} chains one after another, 1 forward solve per step, "
                              f"random walk on the identified coordinates with the refined "
                              f"Laplace covariance, symmetry axis redrawn from its prior "
                              f"conditional, step adapted in burn-in",
                      chains=plain_chains, steps_per_chain=int(draws.shape[0]),
                      burn_per_chain=plain_burn, accept=float(acc_sum / acc_n),
                      burn_seconds=r1.history["burn_seconds"],
                      ms_per_solve=1e3 * post1.seconds / max(post1.solves, 1), **d_plain),
        "pipeline": dict(sampler=f"delayed acceptance, tangent surrogate (affine + second order "
                                 f"along the symmetry axis), {chains} chains x {inner} surrogate "
                                 f"steps per solve (random walk, axis redraws, independence moves "
                                 f"with probability {ind_prob}), invariant coordinates",
                         generations=generations - burn, accept=float(res.result.accept),
                         symmetry_axis="redrawn from its prior conditional inside the surrogate chain",
                         stage1_accept=float(res.result.history["stage1_accept"]),
                         stage2_accept=float(res.result.history["stage2_accept"]),
                         setup_seconds=res.setup_seconds, burn_seconds=res.burn_seconds,
                         solver_seconds_all_generations=res.solver_seconds,
                         surrogate_seconds_all_generations=res.surrogate_seconds,
                         **d_pipe),
        "reference_posterior": dict(sampler="the pipeline's delayed acceptance, fresh chains, "
                                            f"{chains} chains x {ref_generations} generations",
                                    mean_theta=ref_mean.tolist(), sd_theta=ref_sd.tolist(),
                                    rhat=mcmc.rhat(lc.to_u(lc.to_theta(rr.samples[burn:]))).tolist()),
        "mean_check": {"pipeline": mean_check(th), "plain": mean_check(th_plain)},
    }
    for k in ("identified", "symmetry_axis", "all"):
        a, b = d_pipe[f"ess_per_s_{k}"], d_plain[f"ess_per_s_{k}"]
        out[f"ess_per_s_ratio_{k}"] = a / b if b > 0 else None
    out["population_kernel"] = h.population_variant_name(variant)
    if mala_steps > 0:
        post_m = mcmc.Posterior(h, an.L, dt0, prior, checkpoint_every=50)
        lcm = mcmc.LogCoords(post_m, A=mcmc.INVARIANT_MAP)
        v0 = start_points(64, 1.0)
        rm = mcmc.mala(lcm, v0, mala_burn + mala_steps, 0.8, rng, burn=mala_burn,
                       chol=np.linalg.cholesky(res.cov))
        t_m = rm.seconds * mala_steps / (mala_burn + mala_steps)
        d_m = diagnostics(lc.to_theta(rm.samples[mala_burn:]), t_m)
        out["mala"] = dict(sampler="preconditioned MALA (refined Laplace covariance), 64 chains, adjoint "
                                   "gradients with checkpoints every 50 steps, invariant coordinates",
                           steps=mala_steps, burn=mala_burn, accept=float(rm.accept), eps=float(rm.step),
                           ms_per_step=1e3 * rm.seconds / (mala_burn + mala_steps),
                           mean_check=mean_check(lc.to_theta(rm.samples[mala_burn:])), **d_m)
    if unet:
        out["learned_surrogate"] = ls = unet_screen(h, an, prior, dt0, res, rng, train_n=unet_train,
                                                    epochs=unet_epochs)
        # what the trained network gains: the same delayed-acceptance sampler
        # with the network as its screen, against the tangent screen and
        # against no screen (the plain chains)
        out["screen_gain"] = {"identified_ess_per_s": {
            "learned_screen": ls["da_identified_ess_per_s"],
            "tangent_screen": d_pipe["ess_per_s_identified"],
            "no_screen_plain": d_plain["ess_per_s_identified"]},
            "stage2_accept": {"learned_screen": ls["da_stage2_accept"],
                              "tangent_screen": float(res.result.history["stage2_accept"])}}
    h.close()
    return out


def unet_screen(h, an, prior, dt0, res, rng, train_n=20000, epochs=3, gens=20, inner=8):
    """The bf16 U-Net as the stage-1 screen: trained by the library's
    kernels on `train_n` prior draws (batched solver targets), then its
    held-out density error, its log-posterior error near the mode, and the
    stage-2 acceptance of the same delayed-acceptance sampler with it in
    place of the affine surrogate."""
    from gliomauq_gb300 import _lib, mcmc, synthetic as Syn
    lo = (Syn.PRIOR_DW_CM2[0], Syn.PRIOR_RHO[0], Syn.PRIOR_T[0])
    hi = (Syn.PRIOR_DW_CM2[1], Syn.PRIOR_RHO[1], Syn.PRIOR_T[1])
    sg = _lib.Surrogate(h, an.L, lo, hi, batch_max=64, seed=7)
    try:
        train = [p.as_tuple() for p in Syn.draw_prior(an, train_n, seed=21)]
        t0 = time.perf_counter()
        loss = sg.train(train, epochs=epochs, batch=8, lr=1e-3, seed=1)
        t_train = time.perf_counter() - t0
        test = [p.as_tuple() for p in Syn.draw_prior(an, 16, seed=22)]
        pred = sg.loglik(test, want_phi=True)["phi"]
        true = h.batch_solve(test, an.L, with_loglik=False, want_phi=True)["phi"]
        dens = float(np.linalg.norm(pred - true) / np.linalg.norm(true))
        post = mcmc.LogCoords(mcmc.Posterior(h, an.L, dt0, prior), A=mcmc.INVARIANT_MAP)
        Lc = np.linalg.cholesky(res.cov)
        near = res.v_map + rng.standard_normal((64, 6)) @ Lc.T
        near = near[np.isfinite(post.prior.logp(near))]
        exact, _ = post.loglik(near, False)
        sp = post.surrogate(mcmc.SurrogatePosterior(sg, prior))
        t0 = time.perf_counter()
        approx = sp.logpost(near)
        t_eval = (time.perf_counter() - t0) / len(near)
        aff = mcmc.AffineSurrogate(post, res.v_map, 0.5 * np.sqrt(np.diag(res.cov)), quad_axis=0)
        aff_err = float(np.std(exact - aff.logpost(near)))
        t0 = time.perf_counter()
        r = mcmc.da(post, sp, near, gens, 2.38 / np.sqrt(6), rng, inner=inner, burn=0, chol=Lc)
        t_da = time.perf_counter() - t0
        v = r.samples  # the chains' draws in the invariant coordinates
        moved = float(np.mean(np.any(v[1:] != v[:-1], axis=2))) if len(v) > 1 else 0.0
        return {"params": sg.nparams(), "train_samples": train_n, "epochs": epochs,
                "da_seconds": t_da, "da_fraction_of_chain_steps_that_moved": moved,
                "da_identified_ess_per_s": float(mcmc.ess(v)[1:].min() / t_da) if moved > 0 else 0.0,
                "train_seconds": t_train, "train_loss": loss, "heldout_density_rel_l2": dens,
                "seconds_per_eval": t_eval,
                "logpost_error_sd_near_mode": float(np.std(exact - approx)),
                "affine_logpost_error_sd_near_mode": aff_err,
                "exact_logpost_sd_near_mode": float(np.std(exact)),
                "da_stage2_accept": float(r.history["stage2_accept"]),
                "da_generations": gens}
    finally:
        sg.close()


def amr_measurement(device, level=4, steps=20, err_steps=60):
    """The multiresolution-grid kernels (gbg_amr_*) at the size of the
    adaptive configuration: 16^3 blocks of 16^3 cells (256^3), in both exact
    modes (FP64, and the reference's default FP32 storage) and the fast FP32
    mode. All blocks sit
    at one level, with periodic same-level ghost tables (grids with
    resolution jumps take MRAG's own tables); the step evaluates every ghost
    through the tables like any grid. Reports cell-steps/s, algorithmic
    GB/s and the FP32 modes' density error against FP64 after err_steps."""
    from gliomauq_gb300 import _lib, amr, synthetic as Syn
    n = 16 << level
    an = Syn.make_anatomy(n, seed=0)
    phi = np.clip(Syn.gaussian_ic(an, n / 2 + 0.3, n / 2 - 0.6, n / 2 + 0.2, peak=0.1, sigma=1.0), 0, 1)
    L = n * 0.1
    Dw_cm2, rho = 0.0013, 0.025
    Dw = Dw_cm2 / L ** 2
    Dg = 0.1 * Dw
    dt = 0.99 * (1.0 / n) ** 2 / (6.0 * Dw)
    blocks = amr.uniform_blocks(level)
    tables = amr.same_level_ghosts(blocks)
    pw, pg = amr.to_block_major(an.p_w, level), amr.to_block_major(an.p_g, level)
    out = {"grid": f"{len(blocks)} blocks of 16^3 at level {level} ({n}^3), periodic "
                   f"same-level ghost tables", "steps_timed": steps}
    fields = {}
    for mode in ("f64", "f32ref", "f32", "f32_separate"):
        real = 8 if mode == "f64" else 4
        d, g = (Dw, Dg) if mode == "f64" else (float(np.float32(Dw)),
                                               float(np.float32(np.float32(0.1) * np.float32(Dw))))
        with _lib.AmrHandle(len(blocks), "f32" if mode == "f32_separate" else mode, device=device) as h:
            if mode == "f32_separate":
                h.set_fast_variant(1)
            h.set_grid(blocks, pw, pg, amr.to_block_major(phi, level))
            h.set_ghosts(*tables)
            h.step(d, g, rho, dt, 2)
            h.sync()
            t0 = time.perf_counter()
            h.step(d, g, rho, dt, steps)
            h.sync()
            sec = time.perf_counter() - t0
            h.step(d, g, rho, dt, err_steps - 2 - steps)
            fields[mode] = amr.from_block_major(h.get_phi(), level)
        cells = len(blocks) * 4096
        # per cell-step: phi read + write and the cell's tables (exact modes:
        # brain sum and six double face diffusivities; fast mode with a
        # separate ghost pass: six float face coefficients and the mask); per
        # ghost (1736 per block): source value, weight (double), source block
        # and cell (int), CSR start (long), ghost write and read. The fused
        # fast mode: per-face floats (3 x 17/16 per cell), a mask byte, and
        # per ghost a 32-bit start, source index, float weight and the
        # source value, no ghost array.
        if mode == "f32":
            per_cell = 2 * real + 3 * 4 * 17 / 16 + 1 + (1736 / 4096) * (4 + 4 + 4 + 4)
        else:
            tab_bytes = 7 * 4 if mode == "f32_separate" else real + 48
            per_cell = 2 * real + tab_bytes + (1736 / 4096) * (real + 8 + 4 + 4 + 8 + real)
        rate = cells * steps / sec
        out[mode] = {"cell_steps_per_s": rate, "seconds_per_step": sec / steps,
                     "algorithmic_bytes_per_cell_step": per_cell,
                     "algorithmic_gb_per_s": rate * per_cell / 1e9}
    b = fields["f64"]
    out["f32_fused_equals_separate"] = bool(np.array_equal(fields["f32"], fields["f32_separate"]))
    for mode in ("f32ref", "f32"):
        out[f"{mode}_vs_f64_rel_l2"] = float(np.linalg.norm(fields[mode] - b) / np.linalg.norm(b))
    out["error_after_steps"] = err_steps
    return out


def amr_adaptive_measurement(device, level=4, seed=7, steps_per_regrid=20):
    """The adaptive configuration: the seeded anatomy at effective 256^3
    (16^3 blocks at level 4, the maximum level), one prior draw (Dw, rho,
    seed point, T), the Glioma_HG_UQ::run loop on the library's block grid
    with a regrid (one refinement pass at 1e-4, compression at 1e-5 until it
    stops) every `steps_per_regrid` steps and the refinement after the loop
    (gbg_amr_run), in FP64 (exact) and the fast FP32 mode. Reports each
    mode's wall time, cell-steps/s over the steps, regrid seconds per call,
    the range of block counts, and the FP32 run's relative L2 error against
    FP64 on the uniform 256^3 resample."""
    from gliomauq_gb300 import _lib, amr, synthetic as Syn
    n = 16 << level
    an = Syn.make_anatomy(n, seed=0)
    p = Syn.draw_prior(an, 1, seed=seed)[0]
    dt = Syn.reference_dt(n, p.Dw, an.L)[0]
    phi0 = Syn.gaussian_ic(an, p.x0, p.y0, p.z0).astype(np.float32).astype(np.float64)
    blocks = amr.uniform_blocks(level)
    fields = [amr.to_block_major(x, level) for x in (an.p_w, an.p_g, phi0)]
    out = {"config": f"effective {n}^3, 16^3 blocks, levels <= {level}, refine 1e-4, compress "
                     f"1e-5, regrid every {steps_per_regrid} steps",
           "sample": list(p.as_tuple())}
    dumps = {}
    for mode in ("f64", "f32"):
        with _lib.AmrHandle(len(blocks), mode, device=device) as h:
            h.set_grid(blocks, *fields)
            t0 = time.perf_counter()
            steps, regrids = h.run(p.Dw, p.rho, p.T, an.L, bpd=1 << level,
                                   dumpfreq=steps_per_regrid * dt, adaptive=True, max_level=level)
            wall = time.perf_counter() - t0
            st = h.last_run_stats()
            dumps[mode] = h.dump_uniform(n, reference_rules=False)
            lv = h.blocks()[:, 0]
        out[mode] = {"steps": steps, "regrids": regrids, "seconds": wall,
                     "cell_steps_per_s": st["cell_steps"] / st["step_seconds"],
                     "step_seconds": st["step_seconds"],
                     "regrid_ms_per_call": 1e3 * st["regrid_seconds"] / max(1, st["regrid_calls"]),
                     "blocks_min_max": [st["min_blocks"], st["max_blocks"]],
                     "final_levels": {int(k): int(v) for k, v in zip(*np.unique(lv, return_counts=True))}}
    b = dumps["f64"]
    out["f32_vs_f64_rel_l2"] = float(np.linalg.norm(dumps["f32"] - b) / np.linalg.norm(b))
    return out


def c1_measurement(device, n=64, reps=5, lik_reps=50):
    """The plain forward solve of the CPU-runnable configuration (uniform
    64^3, 1 mm voxels, Dw = 0.13 mm^2/day, Dg = Dw/10, rho = 0.025/day,
    Gaussian seed of peak 0.1 and sigma 1 voxel, T = 300 days, the
    reference's dt rule and loop) as one solve per call: the GPU's FP64
    (bit-identical to the reference) and fast FP32 paths, and 512 such solves
    at once on the batched solver; beside them, on the host cores, the
    oracle's FP64 restatement of the reference step and its block-lab port
    (the reference's FP32 default), one whole solve each. Then likelihood
    evaluations per second (HGG_Likelihood: stepPet 3, stepTi 2, selective
    points): gbg_loglik on the GPU-resident field against the oracle's
    restatement on the host."""
    from gliomauq_gb300 import _lib, synthetic as Syn
    from oracle import oracle
    an = Syn.make_anatomy(n, seed=0)
    Dw, rho, T = 0.0013, 0.025, 300.0
    c = (n / 2 + 0.3, n / 2 - 0.6, n / 2 + 0.2)
    phi0 = Syn.gaussian_ic(an, *c, peak=0.1, sigma=1.0)
    dt, dw, dg = Syn.reference_dt(n, Dw, an.L)
    steps = Syn.num_steps(dt, T)
    cells = float(n ** 3 * steps)
    out = {"grid": n, "steps": steps, "cell_steps_per_solve": cells}
    cores = os.cpu_count() or 1
    for prec in ("f64", "f32"):
        h = _lib.Handle(n, prec, device=device)
        try:
            h.set_anatomy(an.p_w, an.p_g)
            t_, d, g = Syn.reference_dt(n, Dw, an.L, f32=(prec == "f32"))
            k_ = Syn.num_steps(t_, T)
            h.set_phi(phi0)
            h.rd_step(d, g, rho, t_, k_)  # warm-up
            t0 = time.perf_counter()
            for _ in range(reps):
                h.set_phi(phi0)
                h.rd_step(d, g, rho, t_, k_)
                u = h.get_phi()
            sec = (time.perf_counter() - t0) / reps
            out[f"gpu_{prec}"] = {"solves_per_s": 1.0 / sec, "cell_steps_per_s": n ** 3 * k_ / sec,
                                  "note": "one solve per call: upload, steps, download"}
            if prec == "f64":
                obs = Syn.make_observations(u, an, seed=3, centre_xyz=c, radius_vox=27.0 * n / 128)
                h.set_observations(obs.pet, obs.t1, obs.t2, obs.points, LIK, step_pet=3, step_ti=2)
                h.loglik()
                t0 = time.perf_counter()
                for _ in range(lik_reps):
                    h.loglik()
                gl = lik_reps / (time.perf_counter() - t0)
                t0 = time.perf_counter()
                for _ in range(5):
                    oracle.loglik(u, obs.pet, obs.t1, obs.t2, obs.points, LIK, 3, 2, True)
                cl = 5 / (time.perf_counter() - t0)
                out["likelihood_evals_per_s"] = {"gpu": gl, "cpu_port_1_thread": cl,
                                                 "note": "gbg_loglik on the resident field, result "
                                                         "copied to the host per call"}
        finally:
            h.close()
    hb = _lib.Handle(n, "f32", device=device, max_samples=512)
    try:
        hb.set_anatomy(an.p_w, an.p_g)
        smp = [(Dw, rho) + c + (T,)] * 512
        hb.batch_solve(smp, an.L, with_loglik=False)
        t0 = time.perf_counter()
        for _ in range(reps):
            hb.batch_solve(smp, an.L, with_loglik=False)
        sec = (time.perf_counter() - t0) / reps
        out["gpu_batched_512_f32"] = {"solves_per_s": 512 / sec, "dense_equivalent_cell_steps_per_s": 512 * cells / sec,
                                      "note": "the skipping kernel computes only tiles that can be nonzero"}
    finally:
        hb.close()
    t0 = time.perf_counter()
    oracle.rd_solve(an.p_w, an.p_g, phi0, dw, dg, rho, dt, steps, "f64", cores)
    sec = time.perf_counter() - t0
    out["cpu_oracle_f64"] = {"solves_per_s": 1.0 / sec, "cell_steps_per_s": cells / sec, "threads": cores}
    d32 = Syn.reference_dt(n, Dw, an.L, f32=True)
    g = oracle.BlockGrid(an.p_w, an.p_g, phi0)
    t0 = time.perf_counter()
    g.steps(d32[1], d32[2], rho, d32[0], steps, cores)
    sec = time.perf_counter() - t0
    out["cpu_blocklab_port_f32"] = {"solves_per_s": 1.0 / sec, "cell_steps_per_s": cells / sec, "threads": cores}
    return out


def graph_measurement(device, n=128, reps=20):
    """gbg_batch_solve per call (host-timed, host buffers in and out) with the
    call as one CUDA graph launch (the default) and as separate kernel
    launches, for a single sample (the plain chain's solve) and for 64 (a
    pipeline generation), prior draws near the truth on the scaled grid."""
    from gliomauq_gb300 import _lib, synthetic as Syn
    an = Syn.make_anatomy(n, seed=0)
    truth = Syn.draw_prior(an, 1, seed=10_000)[0]
    h = _lib.Handle(n, "f32", device=device, max_samples=64)
    out = {}
    try:
        h.set_anatomy(an.p_w, an.p_g)
        u = h.batch_solve([truth.as_tuple()], an.L, with_loglik=False, want_phi=True, dt0=-1.0)["phi"][0]
        obs = Syn.make_observations(u.astype(np.float64), an, seed=3,
                                    centre_xyz=(truth.x0, truth.y0, truth.z0), radius_vox=27.0 * n / 128)
        h.set_observations(obs.pet, obs.t1, obs.t2, obs.points, LIK, step_pet=3, step_ti=2)
        rng = np.random.default_rng(1)
        for S in (1, 64):
            smp = [tuple(np.array(truth.as_tuple()) * (1 + 0.01 * rng.standard_normal(6))) for _ in range(S)]
            res = {}
            for key, graphs in (("graph_ms", True), ("separate_launches_ms", False)):
                h.set_batch_graphs(graphs)
                for _ in range(3):
                    h.batch_solve(smp, an.L, dt0=-1.0)
                t0 = time.perf_counter()
                for _ in range(reps):
                    h.batch_solve(smp, an.L, dt0=-1.0)
                res[key] = 1e3 * (time.perf_counter() - t0) / reps
            out[f"samples_{S}"] = res
    finally:
        h.close()
    return out


def screen_and_statistics_measurement(device, n=128, chains=64, steps=64, reps=3, stat_samples=512):
    """Two kernels of the sampling path at n^3 on the bench problem:
      * the GPU screening chain (k_affine_chain, gbg_affine_chain): `chains`
        chains x `steps` steps of the tangent screen around the truth, ms per
        launch (host-timed call including its small copies) and observation
        points evaluated per second;
      * the propagation statistics (k_field_stats, gbg_field_statistics) of
        `stat_samples` fields of n^3 floats resident in HBM, timed with CUDA
        events on the calling stream, against measured HBM bandwidth on its
        (2 S + 2) * 4 bytes per cell."""
    import torch
    import ctypes as C
    from gliomauq_gb300 import _lib, mcmc, synthetic as Syn
    an = Syn.make_anatomy(n, seed=0)
    truth = Syn.draw_prior(an, 1, seed=10_000)[0]
    h = _lib.Handle(n, "f32", device=device, max_samples=64)
    out = {}
    try:
        h.set_anatomy(an.p_w, an.p_g)
        dt0 = -1.0
        u = h.batch_solve([truth.as_tuple()], an.L, with_loglik=False, want_phi=True, dt0=dt0)["phi"][0]
        obs = Syn.make_observations(u.astype(np.float64), an, seed=3,
                                    centre_xyz=(truth.x0, truth.y0, truth.z0), radius_vox=27.0 * n / 128)
        h.set_observations(obs.pet, obs.t1, obs.t2, obs.points, LIK, step_pet=3, step_ti=2)
        prior = mcmc.Prior.from_anatomy(an)
        lc = mcmc.LogCoords(mcmc.Posterior(h, an.L, dt0, prior), A=mcmc.INVARIANT_MAP)
        v_ref = lc.to_u(np.array([truth.as_tuple()]))[0]
        d = 0.002 * lc.prior.width
        sur = mcmc.AffineSurrogate(lc, v_ref, d, quad_axis=0)
        rng = np.random.default_rng(0)
        v = v_ref + 0.5 * d * rng.standard_normal((chains, 6))
        Lc = np.diag(0.5 * d)
        y, _, _, a1 = sur.chain(v, steps, 1.0, Lc, 0, 0.5, 1)
        t0 = time.perf_counter()
        for r in range(reps):
            y, _, _, a1 = sur.chain(y, steps, 1.0, Lc, 0, 0.5, 2 + r)
        t = (time.perf_counter() - t0) / reps
        npts = int(h.observation_counts()[0] + h.observation_counts()[1])
        out["screen_chain"] = {"kernel": "k_affine_chain", "chains": chains, "steps": steps,
                               "observation_points": npts, "ms_per_launch": 1e3 * t,
                               "us_per_step": 1e6 * t / steps,
                               "points_per_s": chains * steps * npts / t, "random_walk_accept": a1}
    finally:
        h.close()
    gbg = _lib.load()
    dev = torch.device(f"cuda:{device}")
    N = n ** 3
    f = torch.rand((stat_samples, N), dtype=torch.float32, device=dev)
    mean = torch.empty(N, dtype=torch.float32, device=dev)
    var = torch.empty(N, dtype=torch.float32, device=dev)
    st = torch.cuda.current_stream(dev)

    def stats():
        rc = gbg.gbg_field_statistics(n, C.c_void_p(f.data_ptr()), stat_samples, 1, C.c_void_p(mean.data_ptr()),
                                      C.c_void_p(var.data_ptr()), C.c_void_p(st.cuda_stream))
        if rc:
            raise RuntimeError(gbg.gbg_last_error())

    stats()
    torch.cuda.synchronize(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    for _ in range(reps):
        stats()
    e1.record(st)
    torch.cuda.synchronize(dev)
    ms = e0.elapsed_time(e1) / reps
    peak, peak_kind = measured_peaks()
    alg = (2 * stat_samples + 2) * 4.0 * N
    out["field_statistics"] = {"kernel": "k_field_stats", "samples": stat_samples, "grid": n,
                               "ms_per_launch": ms, "algorithmic_bytes": alg,
                               "achieved_gbs": alg / (ms / 1e3) / 1e9, "peak_gbs": peak,
                               "frac": alg / (ms / 1e3) / 1e9 / peak, "peak_source": f"{peak_kind} hbm_gbs",
                               "note": "inputs larger than L2 (the fields are read twice)"}
    del f, mean, var
    torch.cuda.empty_cache()
    return out


def adjoint_measurement(device, n=128, samples=64, reps=2):
    """The discrete adjoint (gbg_adjoint_grad) on the bench problem at n^3:
    forward + gradient and forward only (checkpoints every 50 steps, float
    states, scaled time grid) for `samples` prior draws and for as many
    draws near the truth (1 % perturbations, ~the posterior's step counts),
    beside the batched solve of the same samples; host-timed per call."""
    from gliomauq_gb300 import _lib, synthetic as Syn
    an = Syn.make_anatomy(n, seed=0)
    truth = Syn.draw_prior(an, 1, seed=10_000)[0]
    h = _lib.Handle(n, "f32", device=device, max_samples=max(samples, 1))
    out = {"grid": n, "samples": samples, "checkpoint_every": 50, "time_grid": "scaled (dt0 = -1)"}
    try:
        h.set_anatomy(an.p_w, an.p_g)
        u = h.batch_solve([truth.as_tuple()], an.L, with_loglik=False, want_phi=True, dt0=-1.0)["phi"][0]
        obs = Syn.make_observations(u.astype(np.float64), an, seed=3,
                                    centre_xyz=(truth.x0, truth.y0, truth.z0), radius_vox=27.0 * n / 128)
        h.set_observations(obs.pet, obs.t1, obs.t2, obs.points, LIK, step_pet=3, step_ti=2)
        sets = {"prior": [p.as_tuple() for p in Syn.draw_prior(an, samples, seed=5)],
                "near_mode": [tuple(np.array(truth.as_tuple()) *
                                    (1 + 0.01 * np.random.default_rng(i).standard_normal(6)))
                              for i in range(samples)]}
        for name, smp in sets.items():
            res = {}
            for key, grad in (("forward_and_gradient_ms", True), ("forward_only_ms", False)):
                h.adjoint_grad(smp, -1.0, an.L, checkpoint_every=50, want_grad=grad)
                t0 = time.perf_counter()
                for _ in range(reps):
                    h.adjoint_grad(smp, -1.0, an.L, checkpoint_every=50, want_grad=grad)
                res[key] = 1e3 * (time.perf_counter() - t0) / reps
            h.batch_solve(smp, an.L, dt0=-1.0)
            t0 = time.perf_counter()
            for _ in range(reps):
                r = h.batch_solve(smp, an.L, dt0=-1.0)
            res["batched_solve_ms"] = 1e3 * (time.perf_counter() - t0) / reps
            res["mean_steps"] = float(np.mean(r["nsteps"]))
            res["max_steps"] = int(np.max(r["nsteps"]))
            out[name] = res
    finally:
        h.close()
    return out


def surrogate_measurement(device, n=128, batch=32, reps=5):
    """Forward throughput of the bf16 U-Net surrogate at n^3 (its grid is
    (n/2)^3): milliseconds per sample of gbg_surrogate_loglik (features,
    network, upsampling, likelihood) on each convolution engine, and the
    network's effective TFLOP/s (2 * 27 * Cin * Cout per voxel and layer);
    the same for one training step (loss and parameter gradient)."""
    from gliomauq_gb300 import _lib, synthetic as Syn
    an = Syn.make_anatomy(n, seed=0)
    lo = (Syn.PRIOR_DW_CM2[0], Syn.PRIOR_RHO[0], Syn.PRIOR_T[0])
    hi = (Syn.PRIOR_DW_CM2[1], Syn.PRIOR_RHO[1], Syn.PRIOR_T[1])
    h = _lib.Handle(n, "f32", device=device, max_samples=batch)
    h.set_anatomy(an.p_w, an.p_g)
    truth = Syn.draw_prior(an, 1, seed=10_000)[0]
    u = h.batch_solve([truth.as_tuple()], an.L, with_loglik=False, want_phi=True)["phi"][0]
    obs = Syn.make_observations(u.astype(np.float64), an, seed=3,
                                centre_xyz=(truth.x0, truth.y0, truth.z0), radius_vox=27.0 * n / 128)
    h.set_observations(obs.pet, obs.t1, obs.t2, obs.points, LIK, step_pet=3, step_ti=2)
    sg = _lib.Surrogate(h, an.L, lo, hi, batch_max=batch, seed=7)
    smp = [p.as_tuple() for p in Syn.draw_prior(an, batch, seed=5)]
    m = n // 2
    layers = [(16, 16, m), (16, 16, m), (16, 32, m // 2), (32, 32, m // 2), (32, 32, m // 4),
              (64, 16, m // 2), (32, 16, m), (16, 16, m)]
    flops = float(sum(2 * 27 * ci * co * v ** 3 for ci, co, v in layers))
    out = {"grid": f"{n}^3 (network on {m}^3)", "batch": batch, "params": sg.nparams(),
           "flops_per_sample": flops}
    try:
        for eng in ("tcgen05", "mma.sync"):
            sg.set_engine(eng)
            sg.loglik(smp)
            h.sync()
            t0 = time.perf_counter()
            for _ in range(reps):
                sg.loglik(smp)
            t = (time.perf_counter() - t0) / reps / batch
            out[eng] = {"ms_per_sample": 1e3 * t, "effective_tflops": flops / t / 1e12}
            # one training step (forward, data and weight gradients, loss):
            # three times the forward's convolution flops
            targ = np.random.default_rng(1).uniform(0, 1, (batch, m, m, m)).astype(np.float32)
            sg.loss_grad(smp, targ)
            t0 = time.perf_counter()
            for _ in range(reps):
                sg.loss_grad(smp, targ)
            t = (time.perf_counter() - t0) / reps / batch
            out[eng]["train_step_ms_per_sample"] = 1e3 * t
            out[eng]["train_effective_tflops"] = 3 * flops / t / 1e12
    finally:
        sg.close()
        h.close()
    return out


def reference_arm_observations(an, truth):
    """Observations for the reference arm's likelihood without a GPU: the
    hidden truth solved by the oracle's block-lab port (the reference's FP32
    step) on the host."""
    from gliomauq_gb300 import synthetic as Syn
    from oracle import oracle
    dt, dw, dg = Syn.reference_dt(N, truth.Dw, an.L, f32=True)
    g = oracle.BlockGrid(an.p_w, an.p_g, Syn.gaussian_ic(an, truth.x0, truth.y0, truth.z0))
    g.steps(dw, dg, truth.rho, dt, Syn.num_steps(dt, truth.T), 0)
    u = g.phi().astype(np.float64)
    return Syn.make_observations(u, an, seed=3, centre_xyz=(truth.x0, truth.y0, truth.z0),
                                 radius_vox=27.0)


def run_reference_arm(args):
    rank, _, world = rank_info()
    if rank != 0:
        return
    an, prior, truth = make_workload()
    obs = reference_arm_observations(an, truth)
    vals = []
    for i in range(args.warmup + args.steps):
        b = cpu_baseline(an, prior, seconds=max(2.0, args.ref_seconds), obs=obs)
        if i >= args.warmup:
            vals.append(b["value"])
    v = float(np.mean(vals))
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "solves/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1000.0 * S / v, "ms_per_step_extrapolated": True,
            "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "batched population: 512 forward solves at 128^3 "
                                   "+ per-sample log-likelihood", "n": N, "samples": S},
            "cpu_baseline": dict(b, value=v),
            "e2e": {"value": v, "unit": "solves/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum, one ncu capture
# of the kernel on a 64-sample 128^3 population of the bench's prior) per
# cell-step the kernel computed; traffic grows with the computed cell-steps.
NCU_BYTES_PER_CELL_STEP = {
    "k_population10<": (68.581464e9 + 61.917909e9) / 16350494720.0,
    "k_population8<": 268.869814e9 / 32075939840.0,
}


def computed_cells(h):
    """Cell-steps the latest population launch computed, or None for kernel
    families that do not count them."""
    from gliomauq_gb300 import _lib
    try:
        return h.last_population_cells()
    except _lib.GbgError:
        return None


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gbglioma", choices=["gbglioma", "reference"])
    ap.add_argument("--ref-seconds", type=float, default=8.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-mcmc", action="store_true",
                    help="skip the ESS/s comparison of plain and batched MALA sampling")
    ap.add_argument("--no-amr", action="store_true",
                    help="skip the multiresolution-grid measurement")
    ap.add_argument("--no-surrogate", action="store_true",
                    help="skip the surrogate-network measurement")
    ap.add_argument("--only-surrogate", action="store_true",
                    help="print the surrogate-network measurement alone (profiling runs)")
    ap.add_argument("--only-mcmc", action="store_true",
                    help="print the ESS/s comparison alone")
    ap.add_argument("--only-kernels", action="store_true",
                    help="print the screening-chain and propagation-statistics measurement alone")
    ap.add_argument("--only-amr", action="store_true",
                    help="print the multiresolution-grid measurement alone")
    ap.add_argument("--adjoint-samples", type=int, default=64,
                    help="samples per set in the adjoint measurement")
    ap.add_argument("--only-adjoint", action="store_true",
                    help="print the adjoint measurement alone")
    ap.add_argument("--mcmc-chains", type=int, default=64, help="pipeline chains")
    ap.add_argument("--unet-train", type=int, default=20000,
                    help="prior draws (batched-solver targets) the U-Net screen is trained on")
    ap.add_argument("--unet-epochs", type=int, default=3, help="training passes over them")
    ap.add_argument("--mcmc-seed", type=int, default=0, help="random stream of both samplers")
    ap.add_argument("--mcmc-inner", type=int, default=64, help="surrogate steps per solve")
    ap.add_argument("--mcmc-generations", type=int, default=300,
                    help="pipeline generations (the first 100 are burn-in)")
    ap.add_argument("--mcmc-ind", type=float, default=0.0,
                    help="probability of an independence move per screen step (with the axis "
                         "redraws' 0.5, at most 0.5)")
    ap.add_argument("--mala-steps", type=int, default=0,
                    help="also run the 64-chain adjoint MALA configuration for this many steps")
    ap.add_argument("--samples", type=int, default=S,
                    help="population size (profiling runs use a smaller one)")
    ap.add_argument("--variant", type=int, default=-1,
                    help="population-kernel variant to run (default: the autotuner's choice)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference_arm(args)
    if args.only_surrogate:
        print(json.dumps({"surrogate": surrogate_measurement(int(os.environ.get("LOCAL_RANK", "0")))}))
        return
    if args.only_adjoint:
        print(json.dumps({"adjoint": adjoint_measurement(int(os.environ.get("LOCAL_RANK", "0")),
                                                         samples=args.adjoint_samples)}))
        return
    if args.only_amr:
        dev = int(os.environ.get("LOCAL_RANK", "0"))
        res = amr_measurement(dev)
        res["adaptive"] = amr_adaptive_measurement(dev)
        print(json.dumps({"amr": res}))
        return
    if args.only_kernels:
        dev = int(os.environ.get("LOCAL_RANK", "0"))
        print(json.dumps({"sampling_kernels": screen_and_statistics_measurement(dev),
                          "batch_call": graph_measurement(dev),
                          "c1_plain_solve": c1_measurement(dev)}))
        return
    if args.only_mcmc:
        print(json.dumps({"mcmc": mcmc_comparison(int(os.environ.get("LOCAL_RANK", "0")),
                                                  chains=args.mcmc_chains, inner=args.mcmc_inner,
                                                  generations=args.mcmc_generations,
                                                  unet=not args.no_surrogate,
                                                  mala_steps=args.mala_steps, ind_prob=args.mcmc_ind,
                                                  unet_train=args.unet_train,
                                                  unet_epochs=args.unet_epochs, seed=args.mcmc_seed)}))
        return
    set_population(args.samples)

    import torch
    import torch.distributed as dist

    rank, local_rank, world = rank_info()
    if world > 1:
        dist.init_process_group("nccl", init_method="env://")
    torch.cuda.set_device(local_rank)

    from gliomauq_gb300 import _lib

    an, prior, truth = make_workload(seed_offset=rank)
    per_solve, steps_list = mean_cell_steps(an, prior)
    h = _lib.Handle(N, "f32", device=local_rank, max_samples=S)
    h.set_anatomy(an.p_w, an.p_g)
    tune_cache = os.path.join(ROOT, "gliomauq_gb300", "_build", "tune.json")
    os.makedirs(os.path.dirname(tune_cache), exist_ok=True)
    if args.variant >= 0:
        variant = args.variant
        h.set_population_variant(variant)
    else:
        variant = h.autotune(probe_samples=min(S, 64), cache_path=tune_cache)
    shape = h.population_variants()[variant]
    obs = observations(h, an, truth)
    h.set_observations(obs.pet, obs.t1, obs.t2, obs.points, LIK, step_pet=3, step_ti=2,
                       selective=True)

    samples = np.array([p.as_tuple() for p in prior], dtype=np.float64)
    d_samples = torch.from_numpy(samples).to(f"cuda:{local_rank}")
    d_lik = torch.zeros(S * 5, dtype=torch.float64, device=f"cuda:{local_rank}")
    stream = torch.cuda.ExternalStream(h.stream(), device=f"cuda:{local_rank}")

    def device_step():
        h.batch_solve_device(d_samples.data_ptr(), S, an.L, d_lik.data_ptr())

    torch.cuda.synchronize()
    for _ in range(args.warmup):
        device_step()
    h.sync()

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()
        h.sync()

    # ---- device-resident timed region ----
    clocks = Clocks(local_rank)
    barrier()
    launches0 = h.launch_count()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    pop_ms, pop_cells = [], []
    with torch.cuda.stream(stream):
        ev0.record(stream)
        for _ in range(args.steps):
            device_step()
            pop_ms.append(h.last_population_ms())
            pop_cells.append(computed_cells(h))
        ev1.record(stream)
    barrier()
    launches = h.launch_count() - launches0
    total_ms = ev0.elapsed_time(ev1)
    clk = clocks.stop()
    ms_per_step = max_over_ranks(total_ms, world, f"cuda:{local_rank}") / args.steps
    value = job_rate(S, world, ms_per_step / 1000.0)

    # ---- end to end through the host C ABI ----
    host_samples = [p.as_tuple() for p in prior]
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        res = h.batch_solve(host_samples, an.L, with_loglik=True)
    barrier()
    e2e_s = (time.perf_counter() - t0) / args.steps
    e2e_value = job_rate(S, world, max_over_ranks(e2e_s, world, f"cuda:{local_rank}"))
    assert np.all(res["nsteps"] == np.array(steps_list))
    assert all(np.isfinite(r["total"]) for r in res["loglik"])

    if rank == 0:
        peak, peak_kind = measured_peaks()
        cell_steps = per_solve * S
        dense_bytes = cell_steps * (8.0 + 8.0 / S)
        computed = (float(np.mean(pop_cells)) if all(c is not None for c in pop_cells)
                    else cell_steps)
        # bytes the kernel has to move: the density of every cell-step it
        # computes read and written once, the shared anatomy once per sample
        alg_bytes = computed * (8.0 + 8.0 / S)
        kern_ms = float(np.mean(pop_ms))
        achieved = alg_bytes / (kern_ms / 1000.0) / 1e9
        kname = h.population_variant_name(variant)
        ncu_key = next((k for k in NCU_BYTES_PER_CELL_STEP if kname.startswith(k)), None)
        traffic = NCU_BYTES_PER_CELL_STEP[ncu_key] * computed if ncu_key else None
        line = {
            "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded anatomy, prior draws and observations)",
            "config": {"workload": "batched population: 512 forward solves at 128^3 "
                                   "+ per-sample log-likelihood",
                       "n": N, "samples_per_gpu": S, "mean_steps_per_solve": per_solve / N ** 3,
                       "cell_steps_per_step": cell_steps, "parallelism": f"replicas x{world}",
                       "l2": "inputs larger than L2 (population state 8.6 GB per GPU)",
                       "population_kernel_shape": {"rows_per_tile": shape[0],
                                                   "samples_per_cta": shape[1],
                                                   "threads": shape[2],
                                                   "chosen_by": "gbg_autotune" if args.variant < 0 else "--variant"}},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak,
                         "traffic": traffic,
                         "traffic_source": (
                             f"ncu dram__bytes_read.sum + dram__bytes_write.sum of {ncu_key}...> on a "
                             f"64-sample population of this prior "
                             f"({NCU_BYTES_PER_CELL_STEP[ncu_key]:.3f} B per computed cell-step), "
                             f"scaled by this launch's computed cell-steps" if ncu_key else
                             "no ncu capture of this kernel family"),
                         "kernel": f"{kname} (autotuned variant {variant})",
                         "kernel_ms": kern_ms,
                         "cell_steps_computed": computed,
                         "algorithmic_bytes_per_launch": alg_bytes,
                         "dense_equivalent": {
                             "cell_steps": cell_steps, "bytes": dense_bytes,
                             "achieved": dense_bytes / (kern_ms / 1000.0) / 1e9,
                             "frac": dense_bytes / (kern_ms / 1000.0) / 1e9 / peak,
                             "note": "every cell of every step, as the dense kernels compute it; the "
                                     "skipping kernel leaves out cells that are provably 0"},
                         "peak_source": f"{peak_kind} hbm_gbs"},
            "e2e": {"value": e2e_value, "unit": "solves/s", "h2d_bytes_per_step": 48 * S,
                    "d2h_bytes_per_step": 64 * S + 4},
            "clocks": clk,
            "gpu_launches": int(launches),
        }
        if not args.no_cpu_baseline:
            line["cpu_baseline"] = cpu_baseline(an, prior, obs=obs)
        if not args.no_mcmc:
            line["mcmc"] = mcmc_comparison(local_rank, chains=args.mcmc_chains,
                                           inner=args.mcmc_inner,
                                           generations=args.mcmc_generations,
                                           mala_steps=args.mala_steps, ind_prob=args.mcmc_ind,
                                           unet_train=args.unet_train, unet_epochs=args.unet_epochs)
        if not args.no_amr:
            line["amr"] = amr_measurement(local_rank)
            line["amr"]["adaptive"] = amr_adaptive_measurement(local_rank)
        line["sampling_kernels"] = screen_and_statistics_measurement(local_rank)
        line["batch_call"] = graph_measurement(local_rank)
        line["c1_plain_solve"] = c1_measurement(local_rank)
        line["adjoint"] = adjoint_measurement(local_rank)
        if not args.no_surrogate:
            line["surrogate"] = surrogate_measurement(local_rank)
        print(json.dumps(line))
    h.close()
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
