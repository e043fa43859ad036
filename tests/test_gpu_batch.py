"""GPU: the batched population solver (persistent cooperative kernel) through
the C ABI: per-sample results equal the single-solve fast path bitwise, step
counts follow the reference's time loop, densities stay within the stated
error of the FP64 oracle, and the per-sample likelihood matches the oracle."""
import numpy as np
import pytest

from gliomauq_gb300 import _lib, synthetic as S
from helpers import golden_npz, rel_l2

pytestmark = pytest.mark.gpu

F32_REL_L2_TOL = 1e-5
LIK = (0.0025, 1.0, 0.7, 0.25, 0.09)


def _setup(n=32, seed=4):
    an = S.make_anatomy(n, seed=seed)
    samples = [S.SampleParams(Dw=0.0013, rho=0.025, x0=15.2, y0=16.1, z0=15.7, T=60.0),
               S.SampleParams(Dw=0.0025, rho=0.2, x0=14.0, y0=15.0, z0=16.0, T=25.0),
               S.SampleParams(Dw=0.0002, rho=0.01, x0=16.4, y0=16.6, z0=14.9, T=130.0)]
    return an, samples


def test_batch_equals_single_solve_bitwise(gbg):
    an, samples = _setup()
    n = an.n
    with _lib.Handle(n, "f32", max_samples=len(samples)) as h:
        h.set_anatomy(an.p_w, an.p_g)
        ic = h.batch_solve([s.as_tuple()[:5] + (-1.0,) for s in samples], an.L,
                           with_loglik=False, want_phi=True)
        assert np.all(ic["nsteps"] == 0)
        res = h.batch_solve([s.as_tuple() for s in samples], an.L, with_loglik=False,
                            want_phi=True)
    for i, s in enumerate(samples):
        dt, dw, dg = S.reference_dt(n, s.Dw, an.L)
        assert res["nsteps"][i] == S.num_steps(dt, s.T)
        with _lib.Handle(n, "f32") as h1:
            h1.set_anatomy(an.p_w, an.p_g)
            h1.set_phi(ic["phi"][i].astype(np.float64))
            h1.rd_step(dw, dg, s.rho, dt, int(res["nsteps"][i]))
            single = h1.get_phi()
        assert np.array_equal(single, res["phi"][i].astype(np.float64)), i


def test_batch_initial_condition(gbg):
    an, samples = _setup()
    with _lib.Handle(an.n, "f32", max_samples=3) as h:
        h.set_anatomy(an.p_w, an.p_g)
        ic = h.batch_solve([s.as_tuple()[:5] + (-1.0,) for s in samples], an.L,
                           with_loglik=False, want_phi=True)
    for i, s in enumerate(samples):
        exp = S.gaussian_ic(an, s.x0, s.y0, s.z0).astype(np.float32)
        d = np.abs(ic["phi"][i] - exp)
        assert d.max() <= np.spacing(np.float32(0.1)), d.max()


def test_batch_vs_fp64_oracle_and_loglik(gbg, oracle_lib):
    an, samples = _setup()
    n = an.n
    truth = S.gaussian_ic(an, 15.0, 16.0, 15.0) * 5
    obs = S.make_observations(np.clip(truth, 0, 1), an, seed=3, centre_xyz=(15, 16, 15),
                              radius_vox=9.0)
    with _lib.Handle(n, "f32", max_samples=3) as h:
        h.set_anatomy(an.p_w, an.p_g)
        h.set_observations(obs.pet, obs.t1, obs.t2, obs.points, LIK, step_pet=3, step_ti=2)
        res = h.batch_solve([s.as_tuple() for s in samples], an.L, with_loglik=True,
                            want_phi=True)
    for i, s in enumerate(samples):
        dt, dw, dg = S.reference_dt(n, s.Dw, an.L)
        phi0 = S.gaussian_ic(an, s.x0, s.y0, s.z0).astype(np.float32).astype(np.float64)
        ref = oracle_lib.rd_solve(an.p_w, an.p_g, phi0, dw, dg, s.rho, dt, int(res["nsteps"][i]))
        err = rel_l2(res["phi"][i], ref)
        print(f"sample {i}: steps {res['nsteps'][i]} rel L2 vs FP64 = {err:.3e}")
        assert err <= F32_REL_L2_TOL
        model = res["phi"][i].astype(np.float64)
        o = oracle_lib.loglik(model, obs.pet, obs.t1, obs.t2, obs.points, LIK, 3, 2, True)
        g = res["loglik"][i]
        assert g["n_pet"] == o["n_pet"]
        for k in ("l_pet", "l_t1", "l_t2", "total"):
            assert abs(g[k] - o[k]) <= 1e-11 * max(1.0, abs(o[k]))


def test_batch_argument_errors(gbg):
    an, samples = _setup()
    with _lib.Handle(an.n, "f32", max_samples=2) as h:
        with pytest.raises(_lib.GbgError) as e:
            h.batch_solve([s.as_tuple() for s in samples[:2]], an.L, with_loglik=False)
        assert e.value.status == -5  # anatomy not set
        h.set_anatomy(an.p_w, an.p_g)
        with pytest.raises(_lib.GbgError) as e:
            h.batch_solve([s.as_tuple() for s in samples], an.L, with_loglik=False)  # S > max
        assert e.value.status == -1
        bad = list(samples[0].as_tuple())
        bad[0] = float("nan")
        with pytest.raises(_lib.GbgError) as e:
            h.batch_solve([tuple(bad)], an.L, with_loglik=False)
        assert e.value.status == -4
        with pytest.raises(_lib.GbgError) as e:
            h.batch_solve([samples[0].as_tuple()], an.L, with_loglik=True)  # no observations
        assert e.value.status == -5


@pytest.mark.parametrize("n", [64, 128])
def test_every_population_shape_gives_identical_results(gbg, n):
    """The per-cell arithmetic does not depend on the tile shape or the
    staging (registers, cp.async rings, bulk-copy rings): all population-kernel
    variants agree bitwise."""
    an, samples = _setup(n=n, seed=6)
    c = n / 64.0
    sm = [S.SampleParams(Dw=0.0013, rho=0.03, x0=30.2 * c, y0=33.1 * c, z0=31.5 * c, T=40.0),
          S.SampleParams(Dw=0.0021, rho=0.1, x0=28.0 * c, y0=31.0 * c, z0=33.0 * c, T=25.0),
          S.SampleParams(Dw=0.0009, rho=0.05, x0=33.4 * c, y0=30.6 * c, z0=29.9 * c, T=60.0)]
    with _lib.Handle(n, "f32", max_samples=3) as h:
        h.set_anatomy(an.p_w, an.p_g)
        shapes = h.population_variants()
        assert len(shapes) >= 2
        names = [h.population_variant_name(i) for i in range(len(shapes))]
        assert names[0].startswith(("k_population8<", "k_population10<")), names
        assert len(set(names)) == len(names), names
        with pytest.raises(_lib.GbgError):
            h.population_variant_name(len(shapes))
        outs = []
        for i in range(len(shapes)):
            h.set_population_variant(i)
            outs.append(h.batch_solve([s.as_tuple() for s in sm], an.L, with_loglik=False,
                                      want_phi=True)["phi"])
    for i, o in enumerate(outs[1:], 1):
        assert np.array_equal(o, outs[0]), names[i]


def test_autotune_picks_and_caches(gbg, tmp_path):
    an, samples = _setup()
    cache = str(tmp_path / "tune.json")
    with _lib.Handle(an.n, "f32", max_samples=8) as h:
        h.set_anatomy(an.p_w, an.p_g)
        c1 = h.autotune(probe_samples=8, cache_path=cache)
        assert 0 <= c1 < len(h.population_variants())
        h.set_population_variant(0)
        c2 = h.autotune(probe_samples=8, cache_path=cache)  # served from the cache
        assert c2 == c1
    import json
    with open(cache) as f:
        d = json.load(f)
    assert list(d.values()) == [c1]


@pytest.mark.parametrize("n", [32, 64])
def test_skipping_kernel_equals_dense_on_edge_cases(gbg, n):
    """k_population10 visits only tiles that can be nonzero; its results
    equal the dense default's bit for bit on the cases its bookkeeping has to
    get right: a seed on the brain's boundary layer (masked tissue cells hold
    initial values in round 0 and must be cleared in round 1), a seed outside
    the tissue (empty support), samples of 0, 1 and 2 steps, a wide Gaussian
    whose support box reaches past the faces (periodic wrap), and ordinary
    samples."""
    from helpers import boundary_layer
    an = S.make_anatomy(n, seed=9)
    bl = np.argwhere(boundary_layer(an.brain))  # (z, y, x)
    bz, by, bx = (float(v) for v in bl[len(bl) // 3])
    c = (n - 1) / 2.0
    dt = S.reference_dt(n, 0.0013, an.L)[0]
    smp = [(0.0013, 0.05, bx, by, bz, 30 * dt),          # seed on the boundary layer
           (0.0020, 0.10, -500.0, -500.0, -500.0, 12 * dt),  # far from any tissue: stays 0
           (0.0013, 0.05, c + 0.3, c - 0.2, c, 0.0),      # one step
           (0.0013, 0.05, c - 1.1, c + 0.4, c, 1.5 * dt),  # two steps
           (0.0013, 0.05, c, c, c, -1.0),                 # no step
           (0.0009, 0.12, c + 2.2, c - 3.1, c + 1.7, 40 * dt),
           (0.0024, 0.02, c - 4.0, c + 2.0, c - 1.0, 25 * dt)]
    with _lib.Handle(n, "f32", max_samples=len(smp)) as h:
        h.set_anatomy(an.p_w, an.p_g)
        names = [h.population_variant_name(i) for i in range(len(h.population_variants()))]
        skip = [i for i, nm in enumerate(names) if nm.startswith("k_population10<")]
        dense = [i for i, nm in enumerate(names) if nm.startswith("k_population8<")][0]
        assert skip, names
        for sigma in (1.0, 2.0 * n):
            h.set_population_variant(dense)
            ref = h.batch_solve(smp, an.L, ic_sigma=sigma, with_loglik=False, want_phi=True)
            dense_cells = h.last_population_cells()
            assert dense_cells == int(np.sum(ref["nsteps"])) * n ** 3
            if sigma == 1.0:  # the far seed gives an empty support
                assert not ref["phi"][1].any()
            for i in skip:
                h.set_population_variant(i)
                got = h.batch_solve(smp, an.L, ic_sigma=sigma, with_loglik=False, want_phi=True)
                assert 0 < h.last_population_cells() <= dense_cells
                assert np.array_equal(got["nsteps"], ref["nsteps"])
                for j in range(len(smp)):
                    assert np.array_equal(got["phi"][j], ref["phi"][j]), (names[i], sigma, j)
        assert list(ref["nsteps"][2:5]) == [1, 2, 0]


def test_graph_replay_equals_separate_launches(gbg):
    """gbg_batch_solve as one CUDA graph launch per call: the first call with
    a sample count and options captures the graph, later calls replay it with
    new samples; densities, step counts and log L equal the separately
    launched kernels bit for bit, and a graph is captured anew after the
    observations, the anatomy or the population kernel change."""
    an, samples = _setup()
    n = an.n
    rng = np.random.default_rng(7)
    sets = [[s.as_tuple() for s in samples]]
    for _ in range(2):
        sets.append([(s.Dw * (1 + 0.2 * rng.random()), s.rho * (1 + 0.2 * rng.random()),
                      s.x0 + rng.random(), s.y0 - rng.random(), s.z0, s.T * (0.8 + 0.4 * rng.random()))
                     for s in samples])
    truth = np.clip(S.gaussian_ic(an, 15.0, 16.0, 15.0, peak=0.9, sigma=2.0), 0, 1)
    obs = [S.make_observations(truth, an, seed=sd, centre_xyz=(15, 16, 15), radius_vox=9.0)
           for sd in (3, 5)]

    def solve(h, smp, dt0):
        r = h.batch_solve(smp, an.L, want_phi=True, dt0=dt0)
        return r["phi"], r["nsteps"], np.array([d["total"] for d in r["loglik"]])

    def run(graphs):
        out = []
        with _lib.Handle(n, "f32", max_samples=len(samples)) as h:
            h.set_batch_graphs(graphs)
            h.set_anatomy(an.p_w, an.p_g)
            for o in obs:
                h.set_observations(o.pet, o.t1, o.t2, o.points, LIK, step_pet=1, step_ti=1)
                for smp in sets:
                    for dt0 in (0.0, -1.0):
                        l0 = h.launch_count()
                        out.append(solve(h, smp, dt0) + (h.launch_count() - l0,))
            h.set_population_variant(len(h.population_variants()) - 1)  # the last candidate
            out.append(solve(h, sets[1], 0.0) + (None,))
            h.set_anatomy(an.p_w * 0.5 + an.p_g * 0.5, an.p_g * 0.5 + an.p_w * 0.5)
            out.append(solve(h, sets[2], -1.0) + (None,))
        return out

    eager, graph = run(False), run(True)
    assert len(eager) == len(graph)
    for i, (e, g) in enumerate(zip(eager, graph)):
        assert np.array_equal(e[0], g[0]), i
        assert np.array_equal(e[1], g[1]), i
        assert np.array_equal(e[2], g[2]), i
        if e[3] is not None:
            assert e[3] == g[3], (i, e[3], g[3])
