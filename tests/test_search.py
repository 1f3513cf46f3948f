"""Search drivers (synchronous PSO / DE over whole generations).

CPU tests run the drivers on an analytic fitness; the GPU test runs a few
generations of a particle swarm over the batched FDTD fitness.
"""
from __future__ import annotations

import numpy as np
import pytest

from tomography_gb300 import search as S


def _neg_sphere(centre):
    calls = []

    def f(x):
        calls.append(x.shape)
        return -np.sum((x - centre) ** 2, axis=1)

    return f, calls


@pytest.mark.parametrize("cls", [S.ParticleSwarm, S.DifferentialEvolution])
def test_converges_on_sphere_with_whole_generations(cls):
    lo, hi = np.full(6, -5.0), np.full(6, 5.0)
    centre = np.array([1.0, -2.0, 0.5, 3.0, -1.5, 0.0])
    f, calls = _neg_sphere(centre)
    res = cls(lo, hi, population_size=40, maximum_iterations=150, seed=3).go(f)
    assert res.best_fitness > -1e-3, res.best_fitness
    assert np.all(res.best_params >= lo) and np.all(res.best_params <= hi)
    assert all(c == (40, 6) for c in calls)             # one call per generation, whole population
    assert len(calls) == 151 and res.evaluations == 40 * 151
    assert all(b >= a for a, b in zip(res.history, res.history[1:]))   # best never gets worse


def test_per_candidate_function_and_fixed_bounds():
    """batch=False takes a function of the reference's type (vector -> double);
    a parameter with min == max (test.cxx:70-73, sigma) stays fixed."""
    lo = np.array([1.0, 1.5, 0.0])
    hi = np.array([7.0, 41.0, 0.0])
    seen = []

    def fdtd_like(v):
        assert isinstance(v, list) and len(v) == 3
        seen.append(v[2])
        return -((v[0] - 3.0) ** 2 + (v[1] - 20.0) ** 2)

    res = S.DifferentialEvolution(lo, hi, population_size=12, maximum_iterations=30, seed=5).go(fdtd_like, batch=False)
    assert set(seen) == {0.0}
    assert res.best_fitness > -5.0


def test_arguments_parsed_like_tao():
    argv = ["--population_size", "16", "--maximum_iterations", "3", "--inertia", "0.5", "--seed", "9"]
    ps = S.ParticleSwarm(np.zeros(2), np.ones(2), argv)
    assert (ps.population_size, ps.maximum_iterations, ps.inertia) == (16, 3, 0.5)
    de = S.DifferentialEvolution(np.zeros(2), np.ones(2), ["--parent_selection", "random", "--crossover_rate", "0.9"])
    assert de.parent == "random" and de.cr == 0.9
    with pytest.raises(ValueError):
        S.ParticleSwarm(np.ones(2), np.zeros(2))


def test_same_seed_same_search():
    f, _ = _neg_sphere(np.zeros(4))
    a = S.ParticleSwarm(-np.ones(4), np.ones(4), population_size=10, maximum_iterations=5, seed=11).go(f)
    b = S.ParticleSwarm(-np.ones(4), np.ones(4), population_size=10, maximum_iterations=5, seed=11).go(f)
    assert a.history == b.history
    np.testing.assert_array_equal(a.best_params, b.best_params)


def test_bounds_of_the_reference_search():
    lo, hi = S.reference_bounds()
    assert lo.size == 27 and np.all(hi[18:] == 0) and hi[0] == 7 and hi[9] == 41
    lo, hi = S.breast_bounds(8, 35e-3)
    assert lo.size == 64 and np.all(hi >= lo)


@pytest.mark.gpu
def test_particle_swarm_over_gpu_fitness(tomo):
    from helpers import small_breast_spec, small_params
    from tomography_gb300 import workloads as W

    spec = small_breast_spec(tomo, n_ellipses=2)
    with tomo.Solver(spec.copy(n_ellipses=3)) as ts:
        target = ts.forward(small_params(W, 3), traces=True, far_field=False)["traces"][0]
    lo, hi = S.breast_bounds(2, spec.disc_radius)
    with tomo.Solver(spec) as s:
        s.set_target(target)
        res = S.ParticleSwarm(lo, hi, population_size=8, maximum_iterations=3, seed=1).go(s.fitness_batch)
    assert res.evaluations == 32
    assert np.isfinite(res.best_fitness) and res.best_fitness < 0
    assert all(b >= a for a, b in zip(res.history, res.history[1:]))


@pytest.mark.gpu
def test_search_fitness_over_a_handle(tomo):
    """tomo_search_fitness: the C drivers with the handle's tomo_fitness_batch
    as the generation evaluator.  Same seed, same search as the Python face
    over Solver.fitness_batch; the reported best re-evaluates to its fitness."""
    import ctypes as C

    from helpers import small_breast_spec, small_params
    from tomography_gb300 import workloads as W

    spec = small_breast_spec(tomo, n_ellipses=2)
    with tomo.Solver(spec.copy(n_ellipses=3)) as ts:
        target = ts.forward(small_params(W, 3), traces=True, far_field=False)["traces"][0]
    lo, hi = S.breast_bounds(2, spec.disc_radius)
    lib = tomo.library()
    p = tomo.SearchParams()
    assert lib.tomo_search_defaults(C.byref(p), S.SEARCH_DE) == 0
    p.population_size, p.maximum_iterations, p.seed = 8, 3, 5
    best = np.zeros(lo.size)
    fit = C.c_double()
    hist = np.zeros(4)
    dp = C.POINTER(C.c_double)
    with tomo.Solver(spec) as s:
        s.set_target(target)
        rc = lib.tomo_search_fitness(s._h, C.byref(p), lo.ctypes.data_as(dp), hi.ctypes.data_as(dp), tomo.REPORT_FN(), None,
                                     best.ctypes.data_as(dp), C.byref(fit), hist.ctypes.data_as(dp))
        assert rc == 0, lib.tomo_last_error()
        again = s.fitness(best)
        py = S.DifferentialEvolution(lo, hi, population_size=8, maximum_iterations=3, seed=5).go(s.fitness_batch)
    assert again == fit.value
    assert py.best_fitness == fit.value and list(hist) == py.history
    assert np.all(best >= lo) and np.all(best <= hi)


@pytest.mark.gpu
def test_newton_method_over_gpu_fitness(tomo):
    """The Newton driver over Solver.fitness_batch (test.cxx:116-121's
    anm.iterate(FDTD_GPU) shape): the start point, the regression sample and
    the line search are one batch each; the best point re-evaluates to its
    fitness and is no worse than the start."""
    from helpers import small_breast_spec, small_params
    from tomography_gb300 import workloads as W

    spec = small_breast_spec(tomo, n_ellipses=2)
    with tomo.Solver(spec.copy(n_ellipses=3)) as ts:
        target = ts.forward(small_params(W, 3), traces=True, far_field=False)["traces"][0]
    lo, hi = S.breast_bounds(2, spec.disc_radius)
    sizes = []
    with tomo.Solver(spec) as s:
        s.set_target(target)

        def f(x):
            sizes.append(x.shape[0])
            return s.fitness_batch(x)

        res = S.NewtonMethod(lo, hi, 0.1 * (hi - lo), hessian_diagonal=1, regression_size=40,
                             maximum_iterations=1, seed=3).iterate(f)
        again = s.fitness(res.best_params)
    assert sizes == [1, 40, 13] and res.evaluations == 54
    assert np.isfinite(res.best_fitness) and again == res.best_fitness
    assert res.history[1] >= res.history[0]
    assert np.all(res.best_params >= lo) and np.all(res.best_params <= hi)


def test_search_argument_errors(tomo):
    """tao-style arguments: unknown names are skipped, a malformed value or an
    unknown parent selection is refused; bounds with min > max are refused."""
    import ctypes as C

    lib = tomo.library()
    p = tomo.SearchParams()
    assert lib.tomo_search_defaults(C.byref(p), S.SEARCH_PS) == 0
    assert lib.tomo_search_defaults(C.byref(p), 7) == -1

    def parse(*argv):
        arr = (C.c_char_p * len(argv))(*[a.encode() for a in argv])
        return lib.tomo_search_parse_args(C.byref(p), len(argv), arr)

    assert parse("--population_size", "12", "--unknown", "3", "--inertia", "0.25") == 0
    assert (p.population_size, p.inertia) == (12, 0.25)
    assert parse("--population_size", "12x") == -1
    assert parse("--parent_selection", "worst") == -1
    assert parse("--parent_selection", "random") == 0 and p.parent_best == 0
    lo, hi = np.zeros(2), np.ones(2)
    dp = C.POINTER(C.c_double)
    best, fit = np.zeros(2), C.c_double()
    cb = tomo.BATCH_FN(lambda u, pop, n, npar, out: 0)
    rc = lib.tomo_search_run(C.byref(p), hi.ctypes.data_as(dp), lo.ctypes.data_as(dp), 2, cb, None, tomo.REPORT_FN(), None,
                             best.ctypes.data_as(dp), C.byref(fit), None, None)
    assert rc == -1


CPP_PROGRAM = r"""
#include "tomography_search.hpp"
#include <cstdio>
#include <vector>

static double sphere(const std::vector<double>& v) {    // the reference's fitness type
    double s = 0;
    for (size_t j = 0; j < v.size(); ++j) s += (v[j] - 0.5 * j) * (v[j] - 0.5 * j);
    return -s;
}

int main() {
    std::vector<double> lo(5, -4.0), hi(5, 4.0);
    tomo::ParticleSwarm ps(lo, hi, {"--population_size", "30", "--maximum_iterations", "120", "--seed", "7"});
    int calls = 0;
    tomo::SearchResult a = ps.go([&](const double* pop, size_t n, size_t np, double* fit) {
        ++calls;
        for (size_t i = 0; i < n; ++i) fit[i] = sphere(std::vector<double>(pop + i * np, pop + (i + 1) * np));
    });
    tomo::DifferentialEvolution de(lo, hi, {"--population_size", "30", "--maximum_iterations", "150"});
    tomo::SearchResult b = de.go(sphere);
    tomo::NewtonMethod anm(lo, hi, std::vector<double>(5, 1.0), {"--maximum_iterations", "2"});
    tomo::SearchResult c = anm.iterate(sphere);
    bool threw = false;
    try {
        tomo::ParticleSwarm bad(hi, lo);
        bad.go(sphere);
    } catch (const std::exception&) {
        threw = true;
    }
    std::printf("%d %lld %zu %.9g %.9g %d %.9g\n", calls, (long long)a.evaluations, a.history.size(), a.best_fitness,
                b.best_fitness, threw ? 1 : 0, c.best_fitness);
    return 0;
}
"""


def test_cpp_drivers_have_the_tao_call_shape(tomo, tmp_path):
    """A C++ caller constructs the drivers as tao's are constructed in
    test.cxx:82-121 (bounds, radius, argument strings) and calls go() /
    iterate() with a batch lambda or with a function of the reference's
    fitness type."""
    import os
    import shutil
    import subprocess

    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    repo = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    lib_dir = os.path.dirname(tomo.LIB_PATH)
    src = tmp_path / "search.cpp"
    src.write_text(CPP_PROGRAM)
    exe = tmp_path / "search"
    subprocess.run([cxx, "-std=c++17", "-O1", "-I", os.path.join(repo, "include"), str(src), "-o", str(exe),
                    "-L", lib_dir, "-ltomography_gb300", "-Wl,-rpath," + lib_dir], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()
    calls, evals, nhist = int(out[0]), int(out[1]), int(out[2])
    assert calls == 121 and evals == 30 * 121 and nhist == 121
    assert float(out[3]) > -1e-3 and float(out[4]) > -1e-2
    assert out[5] == "1"   # min > max bounds rejected
    assert float(out[6]) > -1e-9   # the Newton method solves the quadratic


def test_newton_method_solves_a_quadratic_in_one_step():
    """On a concave quadratic the regression model is exact, so the first
    Newton step (line-search multiple 1) lands on the optimum."""
    lo, hi = np.full(5, -5.0), np.full(5, 5.0)
    t = np.array([1.0, -2.0, 0.5, 3.0, -1.5])
    w = np.array([1.0, 2.0, 0.5, 3.0, 1.5])
    calls = []

    def f(x):
        calls.append(x.shape[0])
        return -np.sum(w * (x - t) ** 2, axis=1)

    res = S.NewtonMethod(lo, hi, np.ones(5), line_search_size=4, line_search_min=-1.0, line_search_max=2.0,
                         maximum_iterations=2, seed=1).iterate(f)
    assert res.best_fitness > -1e-9
    np.testing.assert_allclose(res.best_params, t, atol=1e-5)
    # start point, then per iteration one regression batch and one line-search batch
    nu = 1 + 5 + 15
    assert calls == [1, 2 * nu, 4, 2 * nu, 4] and res.evaluations == sum(calls)
    assert all(b >= a for a, b in zip(res.history, res.history[1:]))


def test_newton_method_non_quadratic_fixed_and_diagonal():
    """A quartic objective improves every iteration; a parameter with
    min == max stays fixed (test.cxx:70-73, sigma); the diagonal-Hessian model
    solves a separable quadratic."""
    lo = np.array([-3.0, -3.0, 0.0, -3.0])
    hi = np.array([3.0, 3.0, 0.0, 3.0])
    t = np.array([1.2, -0.7, 0.0, 2.1])
    seen = []

    def quartic(x):
        seen.append(x[:, 2].copy())
        d = x - t
        return -np.sum(d ** 4 + d ** 2, axis=1)

    res = S.NewtonMethod(lo, hi, np.full(4, 0.5), maximum_iterations=8, seed=2).go(quartic)
    assert np.all(np.concatenate(seen) == 0.0)
    assert res.history[-1] > res.history[0] and res.best_fitness > -1e-3
    sep = S.NewtonMethod(lo, hi, np.full(4, 1.0), hessian_diagonal=1, maximum_iterations=1,
                         line_search_size=4).go(lambda x: -np.sum((x - t) ** 2, axis=1))
    assert sep.best_fitness > -1e-9


def test_newton_method_arguments_like_tao():
    argv = ["--maximum_iterations", "3", "--regression_size", "40", "--line_search_size", "5",
            "--line_search_min", "-0.5", "--line_search_max", "1.5", "--hessian_diagonal", "1"]
    nm = S.NewtonMethod(np.zeros(3), np.ones(3), np.full(3, 0.1), argv)
    assert (nm.maximum_iterations, nm.regression_size, nm.line_search_size) == (3, 40, 5)
    assert (nm.line_search_min, nm.line_search_max, nm.hessian_diagonal) == (-0.5, 1.5, 1)
    with pytest.raises(ValueError):
        S.NewtonMethod(np.zeros(3), np.ones(3), np.ones(2))
    bad = S.NewtonMethod(np.zeros(3), np.ones(3), np.ones(3), line_search_size=1)
    with pytest.raises(Exception):
        bad.go(lambda x: -np.sum(x * x, axis=1))


@pytest.mark.parametrize("cls", ["ParticleSwarm", "DifferentialEvolution", "NewtonMethod"])
def test_nan_fitness_ranks_below_every_number(cls):
    """A candidate whose fitness is NaN (a diverged solve) is never kept as
    best, even when it is the first one evaluated."""
    lo, hi = np.full(3, -2.0), np.full(3, 2.0)
    first = [True]

    def f(x):
        v = -np.sum((x - 0.3) ** 2, axis=1)
        if first[0]:
            v[0] = np.nan   # the first candidate of the first batch
            first[0] = False
        v[np.abs(x[:, 1]) > 1.9] = np.nan
        return v

    kw = dict(maximum_iterations=30, seed=5)
    s = (S.NewtonMethod(lo, hi, np.full(3, 0.5), **kw) if cls == "NewtonMethod"
         else getattr(S, cls)(lo, hi, population_size=20, **kw))
    res = s.go(f)
    assert np.isfinite(res.best_fitness) and res.best_fitness > -0.05
    assert np.all(np.isfinite(res.history[1:]))


def test_no_cpp_exception_crosses_the_c_abi(tomo):
    """A host allocation that cannot succeed (a 2^31-member swarm over 10^6
    parameters: 17 PB) returns TOMO_ENOMEM_HOST instead of aborting the
    caller; a full Newton model too large to solve is refused up front."""
    import ctypes as C

    lib = tomo.library()
    p = tomo.SearchParams()
    assert lib.tomo_search_defaults(C.byref(p), S.SEARCH_PS) == 0
    p.population_size, p.maximum_iterations = 2 ** 31 - 1, 1
    n = 10 ** 6
    lo, hi = np.zeros(n), np.ones(n)
    dp = C.POINTER(C.c_double)
    best, fit = np.zeros(n), C.c_double()
    called = []
    cb = tomo.BATCH_FN(lambda u, pop, m, npar, out: called.append(m) or 0)
    rc = lib.tomo_search_run(C.byref(p), lo.ctypes.data_as(dp), hi.ctypes.data_as(dp), n, cb, None, tomo.REPORT_FN(),
                             None, best.ctypes.data_as(dp), C.byref(fit), None, None)
    assert rc == -9 and not called                     # TOMO_ENOMEM_HOST
    assert "allocation" in lib.tomo_last_error().decode()
    with pytest.raises(Exception, match="hessian_diagonal"):
        S.NewtonMethod(np.zeros(200), np.ones(200), np.full(200, 0.1), maximum_iterations=1).go(
            lambda x: -np.sum(x * x, axis=1))
    ok = S.NewtonMethod(np.zeros(200), np.ones(200), np.full(200, 0.1), hessian_diagonal=1, regression_size=450,
                        maximum_iterations=1).go(lambda x: -np.sum((x - 0.5) ** 2, axis=1))
    assert ok.best_fitness > -1e-6
