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
