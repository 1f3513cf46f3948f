"""Synchronous particle-swarm, differential-evolution and regression Newton
drivers over whole generations: Python face of the library's C++ drivers (csrc/search.cpp,
``tomo_search_run`` in include/tomography.h; C++ callers use
include/tomography_search.hpp).

The reference hands its fitness function to tao's searches as a function
pointer (test.cxx:82-121): ``ParticleSwarmMPI ps(min_bound, max_bound,
arguments); ps.go(FDTD_GPU)``, ``DifferentialEvolutionMPI de(...);
de.go(...)``, ``AsynchronousNewtonMethod anm(min_bound, max_bound, radius,
arguments); anm.iterate(FDTD_GPU)``, with tao farming one candidate per MPI
rank and call.  tao itself
is an un-vendored submodule, so the drivers restate the textbook synchronous
algorithms with the same construction and ``go(f)`` call shape, and evaluate
every generation in ONE call: ``f`` receives the whole population as an
``[n, n_param]`` array (``Solver.fitness_batch``), so all candidate x
transmitter solves of a generation advance together on the GPU.  A
per-candidate function of the reference's type (``FDTD_GPU(vector) ->
double``) is accepted too with ``batch=False``.

Fitness is maximised (the reference's fitness is a negative misfit).

Command line (the analogue of the reference's ``--search_type ps|de``)::

    python -m tomography_gb300.search --search_type ps --workload 1 \\
        --population_size 64 --maximum_iterations 20
"""
from __future__ import annotations

import argparse
import ctypes as C
import dataclasses
import json
import sys
import time
from typing import Callable, Sequence

import numpy as np

FitnessFn = Callable[[np.ndarray], np.ndarray]

SEARCH_PS, SEARCH_DE, SEARCH_ANM = 0, 1, 2


from . import BATCH_FN, REPORT_FN, SearchParams  # noqa: E402  (ABI mirrors of include/tomography.h)


@dataclasses.dataclass
class SearchResult:
    best_fitness: float
    best_params: np.ndarray
    history: list            # best fitness after every generation
    evaluations: int         # candidates evaluated
    generations: int
    seconds: float


def get_argument(arguments: Sequence[str] | None, name: str, default, cast=float):
    """``--name value`` from an argv-style list (undvc_common's get_argument shape)."""
    if arguments:
        args = list(arguments)
        for i, a in enumerate(args[:-1]):
            if a == name:
                return cast(args[i + 1])
    return default


class _Search:
    TYPE = SEARCH_PS

    def __init__(self, min_bound, max_bound, arguments=None, *, population_size=None, maximum_iterations=None,
                 seed=None):
        self.lo = np.ascontiguousarray(min_bound, dtype=np.float64)
        self.hi = np.ascontiguousarray(max_bound, dtype=np.float64)
        if self.lo.shape != self.hi.shape or self.lo.ndim != 1:
            raise ValueError("min_bound and max_bound must be equal-length vectors")
        if np.any(self.hi < self.lo):
            raise ValueError("max_bound below min_bound")
        self.n_param = self.lo.size
        self.population_size = int(population_size or get_argument(arguments, "--population_size", 50, int))
        self.maximum_iterations = int(maximum_iterations or get_argument(arguments, "--maximum_iterations", 100, int))
        if self.population_size < 4:
            raise ValueError("population_size must be at least 4")
        self.seed = int(seed if seed is not None else get_argument(arguments, "--seed", 0x70F00001, int))

    def _params(self) -> SearchParams:
        from . import library

        p = SearchParams()
        _check_status(library().tomo_search_defaults(C.byref(p), self.TYPE))
        p.population_size = self.population_size
        p.maximum_iterations = self.maximum_iterations
        p.seed = self.seed & 0xFFFFFFFFFFFFFFFF
        return p

    @staticmethod
    def _evaluator(f, batch: bool) -> FitnessFn:
        if batch:
            def ev(x):
                out = np.asarray(f(np.ascontiguousarray(x)), dtype=np.float64).reshape(-1)
                if out.size != x.shape[0]:
                    raise ValueError(f"fitness function returned {out.size} values for {x.shape[0]} candidates")
                return out
            return ev
        return lambda x: np.array([float(f(list(row))) for row in x], dtype=np.float64)

    def go(self, f, batch: bool = True, callback=None) -> SearchResult:
        """Run the search; ``f`` evaluates a whole generation (``batch=True``)
        or one candidate given as a list (``batch=False``).  ``f`` may be a
        ``Solver``: its batch fitness, with a diverged candidate's non-finite
        fitness ranked below every number instead of raised (the rule of
        ``tomo_search_fitness``)."""
        from . import Solver, library

        if isinstance(f, Solver):
            if f.n_params != self.n_param:
                raise ValueError(f"the solver takes {f.n_params} parameters, the bounds give {self.n_param}")
            solver = f
            f, batch = (lambda x: solver.fitness_batch(x, diverged="keep")), True
        ev = self._evaluator(f, batch)
        errors = []

        def batch_fn(_user, pop, n, npar, out):
            try:
                x = np.ctypeslib.as_array(pop, shape=(n, npar)).copy()
                np.ctypeslib.as_array(out, shape=(n,))[:] = ev(x)
                return 0
            except BaseException as e:   # re-raised after the C driver returns
                errors.append(e)
                return -1

        def report_fn(_user, gen, best, params):
            if callback and not errors:
                try:
                    callback(gen, best, np.ctypeslib.as_array(params, shape=(self.n_param,)).copy())
                except BaseException as e:
                    errors.append(e)

        cb, rep = BATCH_FN(batch_fn), REPORT_FN(report_fn)
        p = self._params()
        best = np.zeros(self.n_param)
        fit = C.c_double()
        hist = np.zeros(self.maximum_iterations + 1)
        evals = C.c_int64()
        dp = C.POINTER(C.c_double)
        t0 = time.perf_counter()
        rc = library().tomo_search_run(C.byref(p), self.lo.ctypes.data_as(dp), self.hi.ctypes.data_as(dp),
                                       self.n_param, cb, None, rep, None, best.ctypes.data_as(dp), C.byref(fit),
                                       hist.ctypes.data_as(dp), C.byref(evals))
        if errors:
            raise errors[0]
        _check_status(rc)
        return SearchResult(float(fit.value), best, [float(h) for h in hist], int(evals.value),
                            self.maximum_iterations, time.perf_counter() - t0)


def _check_status(rc: int) -> None:
    if rc != 0:
        from . import _check

        _check(rc)


class ParticleSwarm(_Search):
    """Synchronous global-best particle swarm.

    v <- w v + c1 r1 (p_best - x) + c2 r2 (g_best - x);  x <- clip(x + v).
    ``--inertia``, ``--local_best_weight``, ``--global_best_weight`` as in tao's
    particle swarm arguments."""

    TYPE = SEARCH_PS

    def __init__(self, min_bound, max_bound, arguments=None, *, inertia=None, local_best_weight=None,
                 global_best_weight=None, **kw):
        super().__init__(min_bound, max_bound, arguments, **kw)
        self.inertia = float(inertia if inertia is not None else get_argument(arguments, "--inertia", 0.75))
        self.c1 = float(local_best_weight if local_best_weight is not None
                        else get_argument(arguments, "--local_best_weight", 1.5))
        self.c2 = float(global_best_weight if global_best_weight is not None
                        else get_argument(arguments, "--global_best_weight", 1.5))

    def _params(self) -> SearchParams:
        p = super()._params()
        p.inertia, p.local_best_weight, p.global_best_weight = self.inertia, self.c1, self.c2
        return p


class DifferentialEvolution(_Search):
    """Synchronous differential evolution, DE/{best,random}/k/bin.

    Donor = parent + F * sum_k (x_a_k - x_b_k) over ``--number_pairs`` pairs of
    distinct other members; binomial crossover at ``--crossover_rate`` with at
    least one donor gene; the trial replaces its target when it is not worse."""

    TYPE = SEARCH_DE

    def __init__(self, min_bound, max_bound, arguments=None, *, crossover_rate=None, differential_scale=None,
                 number_pairs=None, parent_selection=None, **kw):
        super().__init__(min_bound, max_bound, arguments, **kw)
        self.cr = float(crossover_rate if crossover_rate is not None
                        else get_argument(arguments, "--crossover_rate", 0.5))
        self.F = float(differential_scale if differential_scale is not None
                       else get_argument(arguments, "--differential_scale", 0.5))
        self.pairs = int(number_pairs if number_pairs is not None else get_argument(arguments, "--number_pairs", 1, int))
        self.parent = str(parent_selection if parent_selection is not None
                          else get_argument(arguments, "--parent_selection", "best", str))
        if self.parent not in ("best", "random"):
            raise ValueError("parent_selection must be 'best' or 'random'")
        if self.population_size < 2 * self.pairs + 2:
            raise ValueError("population too small for the number of difference pairs")

    def _params(self) -> SearchParams:
        p = super()._params()
        p.crossover_rate, p.differential_scale, p.number_pairs = self.cr, self.F, self.pairs
        p.parent_best = 1 if self.parent == "best" else 0
        return p


class NewtonMethod(_Search):
    """Regression Newton method: each iteration samples ``--regression_size``
    points within ``radius`` of the best point so far (one batch call), fits a
    quadratic model by least squares, and evaluates ``--line_search_size``
    points along the Newton step between ``--line_search_min`` and
    ``--line_search_max`` times the step (one batch call).  The construction
    ``(min_bound, max_bound, radius, arguments)`` and ``iterate(f)`` are those of
    tao's AsynchronousNewtonMethod in the reference's driver (test.cxx:116-121);
    the search starts at the bounds' midpoint.  ``--hessian_diagonal 1`` fits
    only the Hessian's diagonal, for many free parameters."""

    TYPE = SEARCH_ANM

    def __init__(self, min_bound, max_bound, radius=None, arguments=None, *, regression_size=None,
                 line_search_size=None, line_search_min=None, line_search_max=None, hessian_diagonal=None,
                 maximum_iterations=None, seed=None):
        super().__init__(min_bound, max_bound, arguments, population_size=4,
                         maximum_iterations=maximum_iterations or get_argument(arguments, "--maximum_iterations", 10,
                                                                               int), seed=seed)
        self.radius = None if radius is None else np.ascontiguousarray(radius, dtype=np.float64)
        if self.radius is not None and self.radius.shape != self.lo.shape:
            raise ValueError("radius must have one value per parameter")
        self.regression_size = int(regression_size if regression_size is not None
                                   else get_argument(arguments, "--regression_size", 0, int))
        self.line_search_size = int(line_search_size if line_search_size is not None
                                    else get_argument(arguments, "--line_search_size", 13, int))
        self.line_search_min = float(line_search_min if line_search_min is not None
                                     else get_argument(arguments, "--line_search_min", -1.0))
        self.line_search_max = float(line_search_max if line_search_max is not None
                                     else get_argument(arguments, "--line_search_max", 2.0))
        self.hessian_diagonal = int(hessian_diagonal if hessian_diagonal is not None
                                    else get_argument(arguments, "--hessian_diagonal", 0, int))

    def _params(self) -> SearchParams:
        p = super()._params()
        if self.radius is not None:
            p.radius = self.radius.ctypes.data_as(C.POINTER(C.c_double))
        p.regression_size, p.line_search_size = self.regression_size, self.line_search_size
        p.line_search_min, p.line_search_max = self.line_search_min, self.line_search_max
        p.hessian_diagonal = self.hessian_diagonal
        return p

    def iterate(self, f, batch: bool = True, callback=None) -> SearchResult:
        """tao's name for the Newton method's run (``anm.iterate(FDTD_GPU)``)."""
        return self.go(f, batch, callback)


def breast_bounds(n_ellipses: int, disc_radius: float):
    """Per-parameter bounds of the breast-imaging candidates: 8 per ellipse
    (cx, cy, a, b, angle, eps_inf, delta_eps, sigma)."""
    lo = np.tile([-disc_radius, -disc_radius, 2e-3, 2e-3, 0.0, 2.0, 1.0, 0.0], n_ellipses)
    hi = np.tile([disc_radius, disc_radius, 15e-3, 15e-3, np.pi, 20.0, 40.0, 1.0], n_ellipses)
    return lo, hi


def reference_bounds():
    """test.cxx:60-77: eps_inf in [1, 7], delta_eps in [1.5, 41], sigma fixed at 0 for the 3x3 patches."""
    lo = np.array([1.0] * 9 + [1.5] * 9 + [0.0] * 9)
    hi = np.array([7.0] * 9 + [41.0] * 9 + [0.0] * 9)
    return lo, hi


def main(argv=None) -> int:
    argv = list(sys.argv[1:] if argv is None else argv)
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--search_type", required=True, choices=["ps", "de", "anm"])
    ap.add_argument("--workload", type=int, default=1, help="breast-imaging workload (0..4)")
    ap.add_argument("--target_seed_offset", type=int, default=1)
    ap.add_argument("--steps", type=int, default=0, help="override the time steps per solve")
    ap.add_argument("--target", default=None,
                    help="target traces from a file (.npy, .txt/.csv or raw float32; see load_target) instead of "
                         "the workload's synthetic phantom")
    ap.add_argument("--save_target", default=None, help="write the target traces used to this file")
    args, rest = ap.parse_known_args(argv)

    import tomography_gb300 as T
    from tomography_gb300 import workloads as W

    spec = T.breast_spec(args.workload)
    if args.steps:
        spec = spec.copy(steps=args.steps)
    K = spec.n_ellipses
    if args.target:
        target = T.load_target(args.target, spec)
    else:
        with T.Solver(spec.copy(n_ellipses=3)) as ts:
            target = ts.forward(W.target_phantom(args.workload, 3), traces=True, far_field=False)["traces"][0]
    if args.save_target:
        T.save_target(args.save_target, target)
    lo, hi = breast_bounds(K, spec.disc_radius)
    if args.search_type == "anm":
        search = NewtonMethod(lo, hi, 0.1 * (hi - lo), rest)
    else:
        search = (ParticleSwarm if args.search_type == "ps" else DifferentialEvolution)(lo, hi, rest)
    with T.Solver(spec) as s:
        s.set_target(target)

        def report(it, best, _):
            print(json.dumps({"generation": it, "best_fitness": best}), flush=True)

        res = search.go(s, callback=report)
    print(json.dumps({"search_type": args.search_type, "best_fitness": res.best_fitness,
                      "evaluations": res.evaluations, "generations": res.generations, "seconds": res.seconds,
                      "evals_per_s": res.evaluations / res.seconds}))
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
