"""Failure paths, made on the host (no GPU fault, trap or hang is involved).

The reference calls exit(-1) on a CUDA error (FDTD_GPU.cu:35-48), throws
std::out_of_range on a short argument vector (.at(), FDTD_GPU.cu:657-693) and
silently clamps NaN fields to zero (FDTD_GPU.cu:335-350, 425-430).  Here every
failure is a status code:
* a candidate with a non-finite parameter is rejected with TOMO_EINVAL before
  anything is launched (batch and serving paths);
* an unstable candidate (permittivity 0.01: ten times the Courant limit of the
  time step) blows up, and the non-finite detector of the misfit reports
  TOMO_ENUMERIC instead of a fitness;
* a batch above the device-memory budget is refused with TOMO_ENOMEM_BUDGET;
* a fitness without a target is refused with TOMO_ENOTARGET;
and the handle stays usable after each failure: the next valid call returns
the same fitness as on a fresh handle.
"""
from __future__ import annotations

import numpy as np
import pytest

from helpers import small_breast_spec, small_params

pytestmark = pytest.mark.gpu


def _status(tomo, fn, *a):
    try:
        fn(*a)
    except tomo.TomoError as e:
        return e.status
    return 0


def test_failures_are_status_codes_and_the_handle_survives(tomo):
    from tomography_gb300 import workloads as W

    spec = small_breast_spec(tomo, n_ellipses=3, steps=300)
    good = small_params(W, 3, seed_offset=7)
    with tomo.Solver(spec) as s:
        target = s.forward(small_params(W, 3), traces=True, far_field=False)["traces"][0]
    with tomo.Solver(spec) as fresh:
        fresh.set_target(target)
        want = fresh.fitness(good)
    with tomo.Solver(spec) as s:
        assert _status(tomo, s.fitness, good) == -8            # TOMO_ENOTARGET
        s.set_target(target)
        bad = good.copy()
        bad[5] = np.nan                                         # eps_inf of ellipse 0
        assert _status(tomo, s.fitness, bad) == -1              # TOMO_EINVAL, nothing launched
        assert _status(tomo, s.fitness_batch, np.stack([good, bad])) == -1
        assert "non-finite" in tomo.library().tomo_last_error().decode()
        unstable = good.copy()
        unstable[5] = 0.01                                      # 10x the Courant limit of dt
        assert _status(tomo, s.fitness, unstable) == -4         # TOMO_ENUMERIC
        s.set_memory_budget(1)
        assert _status(tomo, s.fitness, good) == -2             # TOMO_ENOMEM_BUDGET
        s.set_memory_budget(0)
        assert s.fitness(good) == want                          # the handle is still usable


def test_poisoned_request_is_rejected_at_submit(tomo):
    from tomography_gb300 import workloads as W

    spec = small_breast_spec(tomo, n_ellipses=3, steps=120)
    good = small_params(W, 3, seed_offset=7)
    bad = good.copy()
    bad[2] = np.inf                                             # semi-axis
    with tomo.Solver(spec) as s:
        target = s.forward(small_params(W, 3), traces=True, far_field=False)["traces"][0]
        s.set_target(target)
        assert _status(tomo, s.submit, np.stack([good, bad])) == -1
        t = s.submit(good)
        got = None
        while got is None:
            s.serve_step()
            got = s.poll(t, 1)
        assert got[0] == s.fitness(good)


def test_search_over_a_handle_ranks_diverged_candidates_last(tomo):
    """tomo_search_fitness goes on past a diverged candidate: its fitness is
    non-finite and ranks below every number.  Ellipse 0 is held at the
    unstable permittivity above (min == max), so every candidate diverges and
    the search ends with TOMO_OK and a best fitness of -infinity; the same
    search with that ellipse stable finds a finite best."""
    import ctypes as C

    from tomography_gb300 import search as S
    from tomography_gb300 import workloads as W

    spec = small_breast_spec(tomo, n_ellipses=3, steps=300)
    good = small_params(W, 3, seed_offset=7)
    lib = tomo.library()
    dp = C.POINTER(C.c_double)
    with tomo.Solver(spec) as s:
        s.set_target(s.forward(small_params(W, 3), traces=True, far_field=False)["traces"][0])
        results = []
        for eps in (0.01, float(good[5])):
            lo, hi = S.breast_bounds(3, spec.disc_radius)
            lo[:8] = hi[:8] = good[:8]
            lo[5] = hi[5] = eps
            p = tomo.SearchParams()
            assert lib.tomo_search_defaults(C.byref(p), S.SEARCH_PS) == 0
            p.population_size, p.maximum_iterations, p.seed = 4, 1, 3
            best, fit = np.zeros(lo.size), C.c_double()
            rc = lib.tomo_search_fitness(s._h, C.byref(p), lo.ctypes.data_as(dp), hi.ctypes.data_as(dp),
                                         tomo.REPORT_FN(), None, best.ctypes.data_as(dp), C.byref(fit), None)
            assert rc == 0, lib.tomo_last_error()
            results.append(fit.value)
        assert results[0] == -np.inf
        assert np.isfinite(results[1])
        assert s.fitness(good) == s.fitness(good)   # the handle is still usable


def test_python_search_over_a_solver_keeps_going(tomo):
    """Solver.fitness_batch(diverged="keep") returns a diverged candidate's
    non-finite fitness beside the others'; a Python search given the Solver
    itself ranks diverged candidates last, as tomo_search_fitness does."""
    from tomography_gb300 import search as S
    from tomography_gb300 import workloads as W

    spec = small_breast_spec(tomo, n_ellipses=3, steps=300)
    good = small_params(W, 3, seed_offset=7)
    unstable = good.copy()
    unstable[5] = 0.01
    with tomo.Solver(spec) as s:
        s.set_target(s.forward(small_params(W, 3), traces=True, far_field=False)["traces"][0])
        with pytest.raises(tomo.TomoError):
            s.fitness_batch(np.stack([good, unstable]))
        f = s.fitness_batch(np.stack([good, unstable]), diverged="keep")
        assert f[0] == s.fitness(good) and not np.isfinite(f[1])
        lo, hi = S.breast_bounds(3, spec.disc_radius)
        lo[:8] = hi[:8] = unstable[:8]
        res = S.ParticleSwarm(lo, hi, population_size=4, maximum_iterations=1, seed=3).go(s)
        assert res.best_fitness == -np.inf and res.evaluations == 8
