"""ctypes binding of libgbglioma.so (include/gbglioma.h).

The library is the product; this module only marshals numpy arrays across
its C ABI. There is no CPU fallback: if the shared library is missing or no
GPU is present, calls raise GbgError.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libgbglioma.so")

GBG_OK = 0
STATUS_NAMES = {0: "OK", -1: "ERR_ARG", -2: "ERR_CUDA", -3: "ERR_TIMEOUT", -4: "ERR_NONFINITE",
                -5: "ERR_STATE", -6: "ERR_NOMEM", -7: "ERR_UNSUPPORTED"}
PREC_F64, PREC_F32REF, PREC_F32 = 0, 1, 2
PREC_BY_NAME = {"f64": PREC_F64, "f32ref": PREC_F32REF, "f32": PREC_F32}

# every symbol the C header declares
EXPORTS = [
    "gbg_create", "gbg_destroy", "gbg_last_error", "gbg_version", "gbg_set_anatomy",
    "gbg_set_phi", "gbg_get_phi", "gbg_rd_step", "gbg_run", "gbg_set_observations",
    "gbg_loglik", "gbg_batch_solve", "gbg_batch_solve_device", "gbg_set_batch_graphs", "gbg_launch_count",
    "gbg_stream", "gbg_sync", "gbg_last_population_ms", "gbg_last_population_cells",
    "gbg_loglik_noalloc",
    "gbg_population_variants", "gbg_set_population_variant", "gbg_population_variant_shape",
    "gbg_autotune", "gbg_amr_create", "gbg_amr_set_grid", "gbg_amr_set_ghosts", "gbg_amr_step",
    "gbg_amr_get_phi", "gbg_amr_fwt_detail", "gbg_adjoint_grad", "gbg_amr_remap",
    "gbg_amr_dump_uniform", "gbg_amr_ghost_tables", "gbg_amr_plan_refine", "gbg_amr_plan_compress",
    "gbg_amr_build_ghosts", "gbg_amr_auto_refine", "gbg_amr_auto_compress", "gbg_amr_get_blocks",
    "gbg_amr_run", "gbg_amr_last_run_stats", "gbg_field_statistics", "gbg_batch_statistics",
    "gbg_surrogate_create", "gbg_surrogate_destroy",
    "gbg_surrogate_nparams", "gbg_surrogate_get_params", "gbg_surrogate_set_params",
    "gbg_surrogate_train", "gbg_surrogate_loss_grad", "gbg_surrogate_features",
    "gbg_surrogate_loglik", "gbg_affine_set", "gbg_affine_loglik", "gbg_affine_set_prior_mask",
    "gbg_affine_chain", "gbg_observation_counts", "gbg_synthetic_observations", "gbg_amr_fast_variant", "gbg_surrogate_set_engine",
    "gbg_set_slopes", "gbg_get_slopes", "gbg_mala_step", "gbg_run_mala",
    "gbg_population_variant_name",
]


class GbgError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


class Config(C.Structure):
    _fields_ = [("n", C.c_int), ("precision", C.c_int), ("device", C.c_int),
                ("max_samples", C.c_int)]


class LikParams(C.Structure):
    _fields_ = [("pet_sigma2", C.c_double), ("pet_scale", C.c_double), ("t1_uc", C.c_double),
                ("t2_uc", C.c_double), ("slope", C.c_double), ("step_pet", C.c_int),
                ("step_ti", C.c_int), ("selective", C.c_int)]


class LikResult(C.Structure):
    _fields_ = [("l_pet", C.c_double), ("l_t1", C.c_double), ("l_t2", C.c_double),
                ("total", C.c_double), ("n_pet", C.c_long)]

    def as_dict(self):
        return dict(l_pet=self.l_pet, l_t1=self.l_t1, l_t2=self.l_t2, total=self.total,
                    n_pet=self.n_pet)


class Sample(C.Structure):
    _fields_ = [("Dw", C.c_double), ("rho", C.c_double), ("x0", C.c_double), ("y0", C.c_double),
                ("z0", C.c_double), ("tend", C.c_double)]


class AdjointOpts(C.Structure):
    _fields_ = [("dt0", C.c_double), ("checkpoint_every", C.c_int), ("L", C.c_double),
                ("ic_peak", C.c_double), ("ic_sigma", C.c_double), ("state_precision", C.c_int)]


class AmrRunOpts(C.Structure):
    _fields_ = [("Dw_file", C.c_double), ("rho", C.c_double), ("tend", C.c_double),
                ("L", C.c_double), ("dumpfreq", C.c_double), ("bpd", C.c_int),
                ("adaptive", C.c_int), ("max_level", C.c_int), ("final_refine", C.c_int),
                ("refine_tol", C.c_double), ("compress_tol", C.c_double)]


class AmrRunStats(C.Structure):
    _fields_ = [("cell_steps", C.c_longlong), ("step_seconds", C.c_double),
                ("regrid_seconds", C.c_double), ("regrid_calls", C.c_int),
                ("min_blocks", C.c_int), ("max_blocks", C.c_int)]


class AmrConfig(C.Structure):
    _fields_ = [("max_blocks", C.c_int), ("precision", C.c_int), ("device", C.c_int)]


class SurrogateConfig(C.Structure):
    _fields_ = [("factor", C.c_int), ("batch_max", C.c_int), ("L", C.c_double),
                ("dw_lo", C.c_double), ("dw_hi", C.c_double), ("rho_lo", C.c_double),
                ("rho_hi", C.c_double), ("t_lo", C.c_double), ("t_hi", C.c_double),
                ("seed", C.c_ulonglong)]


class AffineChainOpts(C.Structure):
    _fields_ = [("axis", C.c_int), ("axis_prob", C.c_double), ("step", C.c_double),
                ("chol", C.c_double * 36), ("u_ref", C.c_double * 6), ("quad_axis", C.c_int),
                ("Ai", C.c_double * 36), ("log_mask", C.c_int), ("lo", C.c_double * 6),
                ("hi", C.c_double * 6), ("ind_prob", C.c_double), ("ind_mean", C.c_double * 6),
                ("ind_chol", C.c_double * 36), ("ind_inv", C.c_double * 36)]


class SyntheticOpts(C.Structure):
    _fields_ = [("uc_t1", C.c_double), ("uc_t2", C.c_double), ("alpha", C.c_double),
                ("seed48", C.c_ulonglong)]


class BatchOpts(C.Structure):
    _fields_ = [("L", C.c_double), ("ic_peak", C.c_double), ("ic_sigma", C.c_double),
                ("with_loglik", C.c_int), ("dt0", C.c_double)]


_lib = None


def load(path: str = LIB_PATH):
    """Load libgbglioma.so and declare its signatures (raises if absent)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise GbgError(-7, f"{path} not built: run gliomauq_gb300.build.build()")
    L = C.CDLL(path)
    vp, dp, fp = C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_float)
    lp = C.POINTER(C.c_long)
    sig = {
        "gbg_create": [C.POINTER(Config), C.POINTER(vp)],
        "gbg_destroy": [vp],
        "gbg_version": [C.POINTER(C.c_int), C.POINTER(C.c_int)],
        "gbg_set_anatomy": [vp, dp, dp],
        "gbg_set_phi": [vp, dp],
        "gbg_get_phi": [vp, dp],
        "gbg_rd_step": [vp, C.c_double, C.c_double, C.c_double, C.c_double, C.c_long],
        "gbg_set_slopes": [vp, dp, dp],
        "gbg_get_slopes": [vp, dp, dp],
        "gbg_mala_step": [vp, C.c_double, C.c_double, C.c_double, C.c_double, C.c_long],
        "gbg_run_mala": [vp, C.c_double, C.c_double, C.c_double, C.c_double, lp, dp],
        "gbg_run": [vp, C.c_double, C.c_double, C.c_double, C.c_double, lp, dp],
        "gbg_set_observations": [vp, dp, dp, dp, dp, C.c_long, C.POINTER(LikParams)],
        "gbg_loglik": [vp, C.POINTER(LikResult)],
        "gbg_batch_solve": [vp, C.POINTER(Sample), C.c_int, C.POINTER(BatchOpts),
                            C.POINTER(LikResult), lp, fp],
        "gbg_batch_solve_device": [vp, C.c_void_p, C.c_int, C.POINTER(BatchOpts), C.c_void_p],
        "gbg_launch_count": [vp, C.POINTER(C.c_longlong)],
        "gbg_stream": [vp, C.POINTER(vp)],
        "gbg_sync": [vp],
        "gbg_last_population_ms": [vp, C.POINTER(C.c_float)],
        "gbg_last_population_cells": [vp, C.POINTER(C.c_longlong)],
        "gbg_population_variants": [vp, C.POINTER(C.c_int)],
        "gbg_set_population_variant": [vp, C.c_int],
        "gbg_set_batch_graphs": [vp, C.c_int],
        "gbg_population_variant_name": [vp, C.c_int, C.c_char_p, C.c_int],
        "gbg_population_variant_shape": [vp, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                         C.POINTER(C.c_int)],
        "gbg_autotune": [vp, C.c_int, C.c_char_p, C.POINTER(C.c_int)],
        "gbg_adjoint_grad": [vp, C.POINTER(Sample), C.c_int, C.POINTER(AdjointOpts), dp, dp],
        "gbg_amr_create": [C.POINTER(AmrConfig), C.POINTER(vp)],
        "gbg_amr_set_grid": [vp, C.c_int, vp, dp, dp, dp],
        "gbg_amr_set_ghosts": [vp, vp, vp, vp, dp, C.c_long],
        "gbg_amr_step": [vp, C.c_double, C.c_double, C.c_double, C.c_double, C.c_long],
        "gbg_amr_get_phi": [vp, dp],
        "gbg_amr_fwt_detail": [vp, dp],
        "gbg_amr_remap": [vp, C.c_int, vp, vp, vp],
        "gbg_amr_dump_uniform": [vp, C.c_int, C.c_int, dp],
        "gbg_amr_ghost_tables": [C.c_int, vp, vp, vp, vp, dp, C.c_long, lp],
        "gbg_amr_plan_refine": [C.c_int, vp, vp, C.c_int, C.c_int, vp, vp, vp,
                                C.POINTER(C.c_int), C.POINTER(C.c_int)],
        "gbg_amr_plan_compress": [C.c_int, vp, vp, C.c_int, vp, vp, vp, C.POINTER(C.c_int),
                                  C.POINTER(C.c_int)],
        "gbg_amr_build_ghosts": [vp],
        "gbg_amr_auto_refine": [vp, C.c_double, C.c_int, C.POINTER(C.c_int)],
        "gbg_amr_auto_compress": [vp, C.c_double, C.POINTER(C.c_int)],
        "gbg_amr_get_blocks": [vp, vp, C.c_int, C.POINTER(C.c_int)],
        "gbg_amr_run": [vp, C.POINTER(AmrRunOpts), lp, C.POINTER(C.c_int)],
        "gbg_amr_last_run_stats": [vp, C.POINTER(AmrRunStats)],
        "gbg_field_statistics": [C.c_int, vp, C.c_int, C.c_int, vp, vp, vp],
        "gbg_batch_statistics": [vp, C.POINTER(Sample), C.c_int, C.POINTER(BatchOpts), C.c_int, dp, dp],
        "gbg_surrogate_create": [vp, C.POINTER(SurrogateConfig), C.POINTER(vp)],
        "gbg_surrogate_destroy": [vp],
        "gbg_surrogate_nparams": [vp, lp],
        "gbg_surrogate_get_params": [vp, fp],
        "gbg_surrogate_set_params": [vp, fp],
        "gbg_surrogate_train": [vp, C.POINTER(Sample), C.c_int, C.c_int, C.c_int, C.c_double,
                                C.c_ulonglong, dp],
        "gbg_surrogate_loss_grad": [vp, C.POINTER(Sample), C.c_int, fp, dp, fp],
        "gbg_surrogate_features": [vp, C.POINTER(Sample), C.c_int, fp],
        "gbg_surrogate_loglik": [vp, C.POINTER(Sample), C.c_int, C.POINTER(LikResult), fp],
        "gbg_surrogate_set_engine": [vp, C.c_int],
        "gbg_affine_set": [vp, C.c_int, fp, fp],
        "gbg_affine_loglik": [vp, C.c_int, dp, C.POINTER(LikResult)],
        "gbg_affine_set_prior_mask": [vp, vp],
        "gbg_observation_counts": [vp, C.POINTER(C.c_long), C.POINTER(C.c_long)],
        "gbg_amr_fast_variant": [vp, C.c_int],
        "gbg_synthetic_observations": [C.c_int, dp, C.c_int, vp, C.POINTER(SyntheticOpts), dp, dp, dp,
                                       C.POINTER(C.c_float)],
        "gbg_affine_chain": [vp, C.POINTER(AffineChainOpts), C.c_int, C.c_int, C.c_ulonglong, dp, dp, dp, vp],
        "gbg_loglik_noalloc": [vp, C.c_int, vp, vp, C.c_long, vp, vp, vp, C.c_long,
                               C.POINTER(LikParams), vp, vp],
    }
    for name, args in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = C.c_int
    L.gbg_last_error.argtypes = []
    L.gbg_last_error.restype = C.c_char_p
    _lib = L
    return L


def check(rc: int):
    if rc != GBG_OK:
        msg = load().gbg_last_error().decode(errors="replace")
        raise GbgError(rc, msg)


def dptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def fptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def as_f64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64)


class Handle:
    """One libgbglioma handle (one CUDA stream, one n^3 grid)."""

    def __init__(self, n: int, precision="f64", device: int = 0, max_samples: int = 0):
        self.lib = load()
        self.n = n
        self.N = n ** 3
        self.max_samples = max_samples
        self.precision = PREC_BY_NAME[precision] if isinstance(precision, str) else precision
        cfg = Config(n, self.precision, device, max_samples)
        h = C.c_void_p()
        check(self.lib.gbg_create(C.byref(cfg), C.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            self.lib.gbg_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _field(self, a):
        a = as_f64(a)
        if a.size != self.N:
            raise ValueError(f"field must have {self.N} cells")
        return a

    def set_anatomy(self, p_w, p_g):
        a, b = self._field(p_w), self._field(p_g)
        check(self.lib.gbg_set_anatomy(self._h, dptr(a), dptr(b)))

    def set_phi(self, phi):
        a = self._field(phi)
        check(self.lib.gbg_set_phi(self._h, dptr(a)))

    def get_phi(self) -> np.ndarray:
        out = np.empty((self.n,) * 3, dtype=np.float64)
        check(self.lib.gbg_get_phi(self._h, dptr(out)))
        return out

    def rd_step(self, Dw, Dg, rho, dt, nsteps=1):
        check(self.lib.gbg_rd_step(self._h, Dw, Dg, rho, dt, nsteps))

    def set_slopes(self, sRho=None, sD=None):
        """MALA variant: the slope fields (None = zero)."""
        a = None if sRho is None else self._field(sRho)
        b = None if sD is None else self._field(sD)
        check(self.lib.gbg_set_slopes(self._h, dptr(a) if a is not None else None,
                                      dptr(b) if b is not None else None))

    def get_slopes(self):
        sr = np.empty((self.n,) * 3, dtype=np.float64)
        sd = np.empty((self.n,) * 3, dtype=np.float64)
        check(self.lib.gbg_get_slopes(self._h, dptr(sr), dptr(sd)))
        return sr, sd

    def mala_step(self, Dw, Dg, rho, dt, nsteps=1):
        check(self.lib.gbg_mala_step(self._h, Dw, Dg, rho, dt, nsteps))

    def run_mala(self, Dw_file, rho, tend, L):
        ns = C.c_long()
        dt = C.c_double()
        check(self.lib.gbg_run_mala(self._h, Dw_file, rho, tend, L, C.byref(ns), C.byref(dt)))
        return ns.value, dt.value

    def run(self, Dw_file, rho, tend, L):
        ns = C.c_long()
        dt = C.c_double()
        check(self.lib.gbg_run(self._h, Dw_file, rho, tend, L, C.byref(ns), C.byref(dt)))
        return ns.value, dt.value

    def set_observations(self, pet, t1, t2, points, params, step_pet=3, step_ti=2,
                         selective=True):
        pet, t1, t2 = self._field(pet), self._field(t1), self._field(t2)
        pts = np.ascontiguousarray(np.asarray(points, dtype=np.float64).T) if selective else None
        npts = pts.shape[1] if pts is not None and pts.size else 0
        lp = LikParams(*params, step_pet, step_ti, 1 if selective else 0)
        check(self.lib.gbg_set_observations(self._h, dptr(pet), dptr(t1), dptr(t2),
                                            dptr(pts) if npts else None, npts, C.byref(lp)))

    def loglik(self) -> dict:
        r = LikResult()
        check(self.lib.gbg_loglik(self._h, C.byref(r)))
        return r.as_dict()

    def batch_solve(self, samples, L, ic_peak=0.1, ic_sigma=1.0, with_loglik=True,
                    want_phi=False, dt0=0.0):
        """dt0 = 0: the reference's time loop per sample; dt0 != 0: the smooth
        time grids of adjoint_grad (dt0 > 0 fixed, dt0 < 0 scaled and stable;
        same forward model, bit for bit)."""
        S = len(samples)
        arr = (Sample * S)(*[Sample(*s) for s in samples])
        opts = BatchOpts(L, ic_peak, ic_sigma, 1 if with_loglik else 0, dt0)
        lik = (LikResult * S)()
        steps = np.zeros(S, dtype=np.int64)
        phi = np.empty((S, self.n, self.n, self.n), dtype=np.float32) if want_phi else None
        check(self.lib.gbg_batch_solve(self._h, arr, S, C.byref(opts),
                                       lik if with_loglik else None,
                                       steps.ctypes.data_as(C.POINTER(C.c_long)),
                                       fptr(phi) if want_phi else None))
        out = dict(nsteps=steps)
        if with_loglik:
            out["loglik"] = [lik[i].as_dict() for i in range(S)]
        if want_phi:
            out["phi"] = phi
        return out

    def batch_statistics(self, samples, L, ic_peak=0.1, ic_sigma=1.0, dt0=0.0,
                         reference_rules=True):
        """Batched solve of the samples, then the per-cell mean and variance of
        their final densities (gbg_batch_statistics): two [z, y, x] arrays."""
        S = len(samples)
        arr = (Sample * S)(*[Sample(*s) for s in samples])
        opts = BatchOpts(L, ic_peak, ic_sigma, 0, dt0)
        mean = np.empty((self.n,) * 3)
        var = np.empty((self.n,) * 3)
        check(self.lib.gbg_batch_statistics(self._h, arr, S, C.byref(opts),
                                            1 if reference_rules else 0, dptr(mean), dptr(var)))
        return mean, var

    def batch_solve_device(self, samples_dev_ptr: int, S: int, L, lik_dev_ptr: int | None,
                           ic_peak=0.1, ic_sigma=1.0, dt0=0.0):
        opts = BatchOpts(L, ic_peak, ic_sigma, 1 if lik_dev_ptr else 0, dt0)
        check(self.lib.gbg_batch_solve_device(self._h, C.c_void_p(samples_dev_ptr), S,
                                              C.byref(opts),
                                              C.c_void_p(lik_dev_ptr) if lik_dev_ptr else None))

    def adjoint_grad(self, samples, dt0, L, ic_peak=0.1, ic_sigma=1.0, checkpoint_every=50,
                     state="f32", want_grad=True):
        """(loglik[S], grad[S, 6]) of the smooth-time-grid forward model;
        grad columns: Dw, rho, x0, y0, z0, tend."""
        S = len(samples)
        arr = (Sample * S)(*[Sample(*s) for s in samples])
        o = AdjointOpts(dt0, checkpoint_every, L, ic_peak, ic_sigma, PREC_BY_NAME[state])
        ll = np.zeros(S)
        g = np.zeros((S, 6))
        check(self.lib.gbg_adjoint_grad(self._h, arr, S, C.byref(o), dptr(ll),
                                        dptr(g) if want_grad else None))
        return ll, (g if want_grad else None)

    def affine_set(self, phi0, J):
        """Affine density model phi0 + sum_p delta_p J[p] (float fields)."""
        p0 = np.ascontiguousarray(phi0, dtype=np.float32).reshape(-1)
        Jf = np.ascontiguousarray(J, dtype=np.float32).reshape(-1, self.N)
        if p0.size != self.N:
            raise ValueError("phi0 must have n^3 values")
        check(self.lib.gbg_affine_set(self._h, Jf.shape[0], fptr(p0), fptr(Jf)))
        self._aff_P = Jf.shape[0]

    def affine_loglik(self, delta) -> np.ndarray:
        """log L totals of the affine models at the rows of delta (B x P)."""
        d = np.ascontiguousarray(np.atleast_2d(delta), dtype=np.float64)
        B = d.shape[0]
        lik = (LikResult * B)()
        check(self.lib.gbg_affine_loglik(self._h, B, dptr(d), lik))
        return np.array([lik[i].total for i in range(B)])

    def observation_counts(self):
        """(PET voxels, T1/T2 points) of the observation lists."""
        a, b = C.c_long(), C.c_long()
        check(self.lib.gbg_observation_counts(self._h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def affine_set_prior_mask(self, mask):
        """The prior's seed-voxel mask ([z, y, x] bool) for affine_chain."""
        m = np.ascontiguousarray(mask, dtype=np.uint8).reshape(-1)
        if m.size != self.N:
            raise ValueError("mask must have n^3 values")
        check(self.lib.gbg_affine_set_prior_mask(self._h, m.ctypes.data))

    def affine_chain(self, v, steps: int, seed: int, *, step: float, chol, axis: int = -1,
                     axis_prob: float = 0.0, u_ref, quad_axis: int = -1, Ai=None, log_mask: int = 0,
                     lo, hi, ind_prob: float = 0.0, ind_mean=None, ind_chol=None):
        """`steps` screening-chain steps for every row of v (B x 6) on the GPU
        (gbg_affine_chain): (v after, log pi* at the start, at the end,
        counts B x 6: random-walk accepts and steps, redraw accepts and
        redraws, independence accepts and proposals). ind_chol: the
        independence Gaussian's factor (row-major, axis decoupled)."""
        vv = np.array(np.atleast_2d(v), dtype=np.float64, order="C", copy=True)
        B = vv.shape[0]
        o = AffineChainOpts()
        o.axis = -1 if axis is None else int(axis)
        o.axis_prob = float(axis_prob)
        o.step = float(step)
        o.chol[:] = np.ascontiguousarray(chol, dtype=np.float64).reshape(36).tolist()
        o.u_ref[:] = np.asarray(u_ref, dtype=np.float64).reshape(6).tolist()
        o.quad_axis = -1 if quad_axis is None else int(quad_axis)
        o.Ai[:] = np.asarray(np.eye(6) if Ai is None else Ai, dtype=np.float64).reshape(36).tolist()
        o.log_mask = int(log_mask)
        o.lo[:] = np.asarray(lo, dtype=np.float64).reshape(6).tolist()
        o.hi[:] = np.asarray(hi, dtype=np.float64).reshape(6).tolist()
        o.ind_prob = float(ind_prob)
        G = np.eye(6) if ind_chol is None else np.asarray(ind_chol, dtype=np.float64).reshape(6, 6)
        o.ind_mean[:] = np.zeros(6).tolist() if ind_mean is None else \
            np.asarray(ind_mean, dtype=np.float64).reshape(6).tolist()
        o.ind_chol[:] = G.reshape(36).tolist()
        o.ind_inv[:] = np.linalg.inv(G).reshape(36).tolist()
        l0 = np.empty(B)
        l1 = np.empty(B)
        cnt = np.zeros((B, 6), dtype=np.int32)
        check(self.lib.gbg_affine_chain(self._h, C.byref(o), B, int(steps),
                                        int(seed) & 0xFFFFFFFFFFFFFFFF, dptr(vv), dptr(l0), dptr(l1),
                                        cnt.ctypes.data))
        return vv, l0, l1, cnt

    def launch_count(self) -> int:
        c = C.c_longlong()
        check(self.lib.gbg_launch_count(self._h, C.byref(c)))
        return c.value

    def stream(self) -> int:
        s = C.c_void_p()
        check(self.lib.gbg_stream(self._h, C.byref(s)))
        return s.value or 0

    def sync(self):
        check(self.lib.gbg_sync(self._h))

    def population_variant_name(self, index: int) -> str:
        buf = C.create_string_buffer(64)
        check(self.lib.gbg_population_variant_name(self._h, index, buf, 64))
        return buf.value.decode()

    def population_variants(self) -> list[tuple[int, int, int]]:
        """(rows per tile, samples per CTA, threads) of every population-kernel shape."""
        c = C.c_int()
        check(self.lib.gbg_population_variants(self._h, C.byref(c)))
        out = []
        for i in range(c.value):
            r, g, t = C.c_int(), C.c_int(), C.c_int()
            check(self.lib.gbg_population_variant_shape(self._h, i, C.byref(r), C.byref(g),
                                                        C.byref(t)))
            out.append((r.value, g.value, t.value))
        return out

    def set_population_variant(self, index: int):
        check(self.lib.gbg_set_population_variant(self._h, index))

    def set_batch_graphs(self, enabled: bool):
        """batch_solve as one CUDA graph launch per call (default) or as
        separate kernel launches; the results are the same bit for bit."""
        check(self.lib.gbg_set_batch_graphs(self._h, 1 if enabled else 0))

    def autotune(self, probe_samples: int = 32, cache_path: str | None = None) -> int:
        c = C.c_int()
        check(self.lib.gbg_autotune(self._h, probe_samples,
                                    cache_path.encode() if cache_path else None, C.byref(c)))
        return c.value

    def last_population_ms(self) -> float:
        ms = C.c_float()
        check(self.lib.gbg_last_population_ms(self._h, C.byref(ms)))
        return ms.value

    def last_population_cells(self) -> int:
        """Cell-steps the latest population-kernel launch computed (tiles
        visited times cells per tile)."""
        c = C.c_longlong()
        check(self.lib.gbg_last_population_cells(self._h, C.byref(c)))
        return c.value


class AmrHandle:
    """A libgbglioma handle on MRAG's multiresolution grid of 16^3 blocks."""

    GHOSTS_PER_BLOCK = 1736

    def __init__(self, max_blocks: int, precision="f64", device: int = 0):
        self.lib = load()
        prec = PREC_BY_NAME[precision] if isinstance(precision, str) else precision
        cfg = AmrConfig(max_blocks, prec, device)
        h = C.c_void_p()
        check(self.lib.gbg_amr_create(C.byref(cfg), C.byref(h)))
        self._h = h
        self.nb = 0

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            self.lib.gbg_destroy(self._h)
            self._h = C.c_void_p()

    __del__ = Handle.__del__
    __enter__ = Handle.__enter__
    __exit__ = Handle.__exit__

    def set_grid(self, blocks, p_w, p_g, phi):
        """blocks: (nb, 4) ints (level, ix, iy, iz); fields: nb*4096 values per field."""
        b = np.ascontiguousarray(blocks, dtype=np.int32)
        nb = b.shape[0]
        f = [as_f64(x).reshape(-1) for x in (p_w, p_g, phi)]
        if any(x.size != nb * 4096 for x in f):
            raise ValueError("fields must have nb*4096 cells")
        check(self.lib.gbg_amr_set_grid(self._h, nb, b.ctypes.data, dptr(f[0]), dptr(f[1]),
                                        dptr(f[2])))
        self.nb = nb

    def set_ghosts(self, start, src_block, src_cell, w):
        st = np.ascontiguousarray(start, dtype=np.int64)
        sb = np.ascontiguousarray(src_block, dtype=np.int32)
        sc = np.ascontiguousarray(src_cell, dtype=np.int32)
        ww = as_f64(w)
        check(self.lib.gbg_amr_set_ghosts(self._h, st.ctypes.data, sb.ctypes.data, sc.ctypes.data,
                                          dptr(ww), int(ww.size)))

    def step(self, Dw, Dg, rho, dt, nsteps=1):
        """Enqueues the steps on the handle's stream (returns before they finish)."""
        check(self.lib.gbg_amr_step(self._h, Dw, Dg, rho, dt, nsteps))

    def set_fast_variant(self, variant: int):
        """Fast FP32 step form: 0 fused ghosts (default), 1 separate ghost pass."""
        check(self.lib.gbg_amr_fast_variant(self._h, variant))

    def sync(self):
        check(self.lib.gbg_sync(self._h))

    def get_phi(self) -> np.ndarray:
        out = np.empty((self.nb, 16, 16, 16), dtype=np.float64)
        check(self.lib.gbg_amr_get_phi(self._h, dptr(out)))
        return out

    def fwt_detail(self) -> np.ndarray:
        out = np.empty(self.nb, dtype=np.float64)
        check(self.lib.gbg_amr_fwt_detail(self._h, dptr(out)))
        return out

    def remap(self, new_blocks, kind, src):
        """Split / collapse / copy into the grid `new_blocks` (see gbg_amr_remap)."""
        b = np.ascontiguousarray(new_blocks, dtype=np.int32)
        k = np.ascontiguousarray(kind, dtype=np.int32)
        s = np.ascontiguousarray(src, dtype=np.int32).reshape(-1, 8)
        check(self.lib.gbg_amr_remap(self._h, b.shape[0], b.ctypes.data, k.ctypes.data,
                                     s.ctypes.data))
        self.nb = b.shape[0]

    def dump_uniform(self, gpd: int, reference_rules: bool = True) -> np.ndarray:
        out = np.empty((gpd, gpd, gpd), dtype=np.float64)
        check(self.lib.gbg_amr_dump_uniform(self._h, gpd, 1 if reference_rules else 0, dptr(out)))
        return out

    def build_ghosts(self):
        """Compile and install the ghost tables of the current blocks."""
        check(self.lib.gbg_amr_build_ghosts(self._h))

    def blocks(self) -> np.ndarray:
        """(nb, 4) ints (level, ix, iy, iz) of the current grid, device order."""
        n = C.c_int()
        check(self.lib.gbg_amr_get_blocks(self._h, None, 0, C.byref(n)))
        out = np.empty((n.value, 4), dtype=np.int32)
        check(self.lib.gbg_amr_get_blocks(self._h, out.ctypes.data, n.value, C.byref(n)))
        self.nb = n.value
        return out

    def auto_refine(self, tol=1e-4, max_level=-1) -> int:
        r = C.c_int()
        check(self.lib.gbg_amr_auto_refine(self._h, tol, max_level, C.byref(r)))
        self.blocks()
        return r.value

    def auto_compress(self, tol=1e-5) -> int:
        c = C.c_int()
        check(self.lib.gbg_amr_auto_compress(self._h, tol, C.byref(c)))
        self.blocks()
        return c.value

    def run(self, Dw_file, rho, tend, L, bpd, dumpfreq=1e30, adaptive=False, max_level=-1,
            final_refine=True, refine_tol=1e-4, compress_tol=1e-5):
        """Glioma_HG_UQ::run on this grid (gbg_amr_run); returns (steps, regrids)."""
        o = AmrRunOpts(Dw_file, rho, tend, L, dumpfreq, bpd, 1 if adaptive else 0, max_level,
                       1 if final_refine else 0, refine_tol, compress_tol)
        steps, regrids = C.c_long(), C.c_int()
        check(self.lib.gbg_amr_run(self._h, C.byref(o), C.byref(steps), C.byref(regrids)))
        self.blocks()
        return steps.value, regrids.value

    def last_run_stats(self) -> dict:
        s = AmrRunStats()
        check(self.lib.gbg_amr_last_run_stats(self._h, C.byref(s)))
        return {k: getattr(s, k) for k, _ in AmrRunStats._fields_}


def synthetic_observations(tumor, block_order=None, uc_t1=0.8, uc_t2=0.3, alpha=0.02, seed48=0):
    """PET, T1, T2 ([z, y, x] float64) and the centre of mass (3 floats) the
    reference's synthetic-data program makes from a tumour density
    (gbg_synthetic_observations); block_order: (level, ix, iy, iz) rows in
    the grid's loop order, None for x fastest."""
    lib = load()
    t = np.ascontiguousarray(tumor, dtype=np.float64)
    n = t.shape[0]
    pet, t1, t2 = (np.empty_like(t) for _ in range(3))
    com = (C.c_float * 3)()
    o = SyntheticOpts(uc_t1, uc_t2, alpha, seed48)
    if block_order is None:
        nb, bp = 0, None
    else:
        b = np.ascontiguousarray(block_order, dtype=np.int32).reshape(-1, 4)
        nb, bp = b.shape[0], b.ctypes.data
    check(lib.gbg_synthetic_observations(n, dptr(t), nb, bp, C.byref(o), dptr(pet), dptr(t1), dptr(t2),
                                         com))
    return pet, t1, t2, np.array(list(com), dtype=np.float32)


def amr_ghost_tables(blocks):
    """Host-only: (start, src_block, src_cell, w) of a periodic block tree
    (gbg_amr_ghost_tables)."""
    lib = load()
    b = np.ascontiguousarray(blocks, dtype=np.int32)
    nb = b.shape[0]
    start = np.empty(nb * AmrHandle.GHOSTS_PER_BLOCK + 1, dtype=np.int64)
    n = C.c_long()
    check(lib.gbg_amr_ghost_tables(nb, b.ctypes.data, start.ctypes.data, None, None, None, 0,
                                   C.byref(n)))
    sb = np.empty(n.value, dtype=np.int32)
    sc = np.empty(n.value, dtype=np.int32)
    w = np.empty(n.value, dtype=np.float64)
    check(lib.gbg_amr_ghost_tables(nb, b.ctypes.data, start.ctypes.data, sb.ctypes.data,
                                   sc.ctypes.data, dptr(w), n.value, C.byref(n)))
    return start, sb, sc, w


def _plan(fn, blocks, flagged, *extra):
    lib = load()
    b = np.ascontiguousarray(blocks, dtype=np.int32)
    nb = b.shape[0]
    f = np.ascontiguousarray(flagged, dtype=np.uint8)
    cap = 8 * nb
    nbk = np.empty((cap, 4), dtype=np.int32)
    kind = np.empty(cap, dtype=np.int32)
    src = np.empty((cap, 8), dtype=np.int32)
    nn, cnt = C.c_int(), C.c_int()
    check(getattr(lib, fn)(nb, b.ctypes.data, f.ctypes.data, *extra, cap, nbk.ctypes.data,
                           kind.ctypes.data, src.ctypes.data, C.byref(nn), C.byref(cnt)))
    return nbk[:nn.value], kind[:nn.value], src[:nn.value], cnt.value


def amr_plan_refine(blocks, flagged, max_level=-1):
    """Host-only: (new blocks, kind, src, refined) of Grid::refine's plan."""
    return _plan("gbg_amr_plan_refine", blocks, flagged, max_level)


def amr_plan_compress(blocks, flagged):
    """Host-only: (new blocks, kind, src, collapses) of Grid::compress's plan."""
    return _plan("gbg_amr_plan_compress", blocks, flagged)


def _samples(samples):
    S = len(samples)
    return S, (Sample * S)(*[Sample(*s) for s in samples])


class Surrogate:
    """bf16 3D U-Net surrogate of the final density, bound to a GBG_PREC_F32
    Handle (its anatomy, observations and batched solver). Destroy it before
    the handle it was created on."""

    def __init__(self, handle: Handle, L: float, prior_lo, prior_hi, batch_max: int = 8,
                 factor: int = 2, seed: int = 1):
        self.lib = handle.lib
        self.handle = handle
        self.m = handle.n // factor
        cfg = SurrogateConfig(factor, batch_max, L, prior_lo[0], prior_hi[0], prior_lo[1],
                              prior_hi[1], prior_lo[2], prior_hi[2], seed)
        self._s = C.c_void_p()
        check(self.lib.gbg_surrogate_create(handle._h, C.byref(cfg), C.byref(self._s)))
        self.batch_max = batch_max

    def close(self):
        if self._s:
            self.lib.gbg_surrogate_destroy(self._s)
            self._s = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def nparams(self) -> int:
        c = C.c_long()
        check(self.lib.gbg_surrogate_nparams(self._s, C.byref(c)))
        return c.value

    def set_engine(self, engine: str):
        """Convolution kernels: "tcgen05" or "mma.sync"."""
        check(self.lib.gbg_surrogate_set_engine(self._s, {"mma.sync": 0, "tcgen05": 1}[engine]))

    def get_params(self) -> np.ndarray:
        p = np.empty(self.nparams(), dtype=np.float32)
        check(self.lib.gbg_surrogate_get_params(self._s, fptr(p)))
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        if p.size != self.nparams():
            raise ValueError("parameter vector has the wrong length")
        check(self.lib.gbg_surrogate_set_params(self._s, fptr(p)))

    def train(self, samples, epochs: int, batch: int, lr: float = 1e-3, seed: int = 0) -> float:
        S, arr = _samples(samples)
        loss = C.c_double()
        check(self.lib.gbg_surrogate_train(self._s, arr, S, epochs, batch, lr, seed,
                                           C.byref(loss)))
        return loss.value

    def loss_grad(self, samples, targets, want_grad=True):
        B, arr = _samples(samples)
        t = np.ascontiguousarray(targets, dtype=np.float32)
        if t.size != B * self.m ** 3:
            raise ValueError("targets must hold B fields of (n/factor)^3 values")
        loss = C.c_double()
        g = np.empty(self.nparams(), dtype=np.float32) if want_grad else None
        check(self.lib.gbg_surrogate_loss_grad(self._s, arr, B, fptr(t), C.byref(loss),
                                               fptr(g) if want_grad else None))
        return loss.value, g

    def features(self, samples) -> np.ndarray:
        B, arr = _samples(samples)
        out = np.empty((B, self.m, self.m, self.m, 16), dtype=np.float32)
        check(self.lib.gbg_surrogate_features(self._s, arr, B, fptr(out)))
        return out

    def loglik(self, samples, want_phi=False):
        B, arr = _samples(samples)
        lik = (LikResult * B)()
        n = self.handle.n
        phi = np.empty((B, n, n, n), dtype=np.float32) if want_phi else None
        check(self.lib.gbg_surrogate_loglik(self._s, arr, B, lik, fptr(phi) if want_phi else None))
        out = dict(loglik=[lik[i].as_dict() for i in range(B)])
        if want_phi:
            out["phi"] = phi
        return out
