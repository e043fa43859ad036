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
           copied in, log-likelihoods and step counts copied out each step)
  roofline: the population kernel's algorithmic bytes (8 B per cell-step of
           state plus 8/S B of shared anatomy) over its event-timed duration,
           against the measured HBM copy bandwidth
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


def cpu_baseline(an, prior, seconds=12.0):
    """The oracle's block-lab restatement of the reference CPU step, all cores,
    on one sample of the workload for about `seconds`; scaled to solves/s."""
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
    return dict(value=cs / per_solve, unit="solves/s", cores=cores, kind="port",
                sample=f"{steps} steps of one 128^3 sample ({el:.1f} s), block-lab restatement "
                       f"of the reference CPU step (FP32 Real, {cores} threads); "
                       f"{cs / 1e6:.1f} Mcell-steps/s scaled by the population's mean "
                       f"{per_solve / N ** 3:.1f} steps per solve")


def mcmc_comparison(device, mala_steps=120, mala_burn=40, rwm_steps=2000, rwm_burn=500,
                    n=64, chains=64):
    """Posterior ESS/s of plain single-solve MCMC (one random-walk chain,
    one forward solve per step) against batched MALA (64 chains, one batched
    forward + adjoint call per generation), same posterior, at n^3."""
    from gliomauq_gb300 import _lib, mcmc, synthetic as Syn
    an = Syn.make_anatomy(n, seed=0)
    truth = Syn.draw_prior(an, 1, seed=10_000)[0]
    rng = np.random.default_rng(0)
    h = _lib.Handle(n, "f32", device=device, max_samples=chains)
    h.set_anatomy(an.p_w, an.p_g)
    u = h.batch_solve([truth.as_tuple()], an.L, with_loglik=False, want_phi=True)["phi"][0]
    obs = Syn.make_observations(u.astype(np.float64), an, seed=3,
                                centre_xyz=(truth.x0, truth.y0, truth.z0),
                                radius_vox=27.0 * n / 128)
    h.set_observations(obs.pet, obs.t1, obs.t2, obs.points, LIK, step_pet=3, step_ti=2)
    prior = mcmc.Prior.from_anatomy(an)
    dt0 = Syn.reference_dt(n, prior.hi[0], an.L)[0]
    th0 = np.array([truth.as_tuple()] * chains) + rng.normal(0, 1e-3, (chains, 6)) * prior.width
    post = mcmc.Posterior(h, an.L, dt0, prior)
    r = mcmc.mala(post, th0, mala_steps, 2e-3, rng, burn=mala_burn)
    t_mala = r.seconds * (mala_steps - mala_burn) / mala_steps
    e_mala = mcmc.ess(r.samples[mala_burn:])
    post1 = mcmc.Posterior(h, an.L, dt0, prior)
    r1 = mcmc.rwm(post1, th0[:1], rwm_steps, 1e-3, rng, burn=rwm_burn)
    t_rwm = r1.seconds * (rwm_steps - rwm_burn) / rwm_steps
    e_rwm = mcmc.ess(r1.samples[rwm_burn:])
    h.close()
    plain = float(e_rwm.min() / t_rwm)
    mala = float(e_mala.min() / t_mala)
    return {"grid": n, "posterior": "synthetic truth, PET/T1/T2 likelihood, smooth-time-grid model",
            "plain": {"sampler": "RWM, 1 chain, 1 forward solve per step", "steps": rwm_steps - rwm_burn,
                      "accept": float(r1.accept), "ess_min": float(e_rwm.min()),
                      "seconds": t_rwm, "ess_per_s": plain},
            "batched_adjoint": {"sampler": f"MALA, {chains} chains, batched forward+adjoint",
                                "steps": mala_steps - mala_burn, "accept": float(r.accept),
                                "ess_min": float(e_mala.min()), "seconds": t_mala,
                                "ess_per_s": mala},
            "ess_per_s_ratio": mala / plain if plain > 0 else None,
            "surrogate": "not built"}


def run_reference_arm(args):
    rank, _, world = rank_info()
    if rank != 0:
        return
    an, prior, _ = make_workload()
    vals = []
    for i in range(args.warmup + args.steps):
        b = cpu_baseline(an, prior, seconds=max(2.0, args.ref_seconds))
        if i >= args.warmup:
            vals.append(b["value"])
    v = float(np.mean(vals))
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "solves/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1000.0 * S / v, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "batched population: 512 forward solves at 128^3 "
                                   "+ per-sample log-likelihood", "n": N, "samples": S},
            "cpu_baseline": dict(b, value=v),
            "e2e": {"value": v, "unit": "solves/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


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
    ap.add_argument("--samples", type=int, default=S,
                    help="population size (profiling runs use a smaller one)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference_arm(args)
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
    pop_ms = []
    with torch.cuda.stream(stream):
        ev0.record(stream)
        for _ in range(args.steps):
            device_step()
            pop_ms.append(h.last_population_ms())
        ev1.record(stream)
    barrier()
    launches = h.launch_count() - launches0
    total_ms = ev0.elapsed_time(ev1)
    clk = clocks.stop()
    t = torch.tensor([total_ms], dtype=torch.float64, device=f"cuda:{local_rank}")
    if world > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    ms_per_step = float(t.item()) / args.steps
    value = world * S / (ms_per_step / 1000.0)

    # ---- end to end through the host C ABI ----
    host_samples = [p.as_tuple() for p in prior]
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        res = h.batch_solve(host_samples, an.L, with_loglik=True)
    barrier()
    e2e_s = (time.perf_counter() - t0) / args.steps
    te = torch.tensor([e2e_s], dtype=torch.float64, device=f"cuda:{local_rank}")
    if world > 1:
        dist.all_reduce(te, op=dist.ReduceOp.MAX)
    e2e_value = world * S / float(te.item())
    assert np.all(res["nsteps"] == np.array(steps_list))
    assert all(np.isfinite(r["total"]) for r in res["loglik"])

    if rank == 0:
        peak, peak_kind = measured_peaks()
        cell_steps = per_solve * S
        alg_bytes = cell_steps * (8.0 + 8.0 / S)
        kern_ms = float(np.mean(pop_ms))
        achieved = alg_bytes / (kern_ms / 1000.0) / 1e9
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
                                                   "chosen_by": "gbg_autotune"}},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": None,
                         "kernel": "k_population2", "kernel_ms": kern_ms,
                         "algorithmic_bytes_per_launch": alg_bytes,
                         "peak_source": f"{peak_kind} hbm_gbs"},
            "e2e": {"value": e2e_value, "unit": "solves/s", "h2d_bytes_per_step": 48 * S,
                    "d2h_bytes_per_step": 64 * S + 4},
            "clocks": clk,
            "gpu_launches": int(launches),
        }
        if not args.no_cpu_baseline:
            line["cpu_baseline"] = cpu_baseline(an, prior)
        if not args.no_mcmc:
            line["mcmc"] = mcmc_comparison(local_rank)
        print(json.dumps(line))
    h.close()
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
