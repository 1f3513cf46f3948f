"""Serving loop: continuous batching with admission by memory budget.

The same request must give bit-identical fitness alone, in a mix with other
requests (admitted while it runs, different progress), and through the
batch path (same kernels, same blocking).
"""
from __future__ import annotations

import numpy as np
import pytest

from helpers import small_breast_spec, small_params

pytestmark = pytest.mark.gpu


def _cands(W, n, seed, k=4):
    return np.stack([W.candidate_params(seed + 1000 * i, k, disc_radius=15e-3) for i in range(n)])


def _drain(solver, tickets, ncands, max_steps=100000):
    done = {}
    for _ in range(max_steps):
        solver.serve_step()
        for t, n in zip(tickets, ncands):
            if t not in done:
                r = solver.poll(t, n)
                if r is not None:
                    done[t] = r
        if len(done) == len(tickets):
            return done
    raise AssertionError("serving loop did not finish")


def _solver(tomo, W, **kw):
    spec = small_breast_spec(tomo, n_ellipses=4, steps=240, **kw)
    s = tomo.Solver(spec)
    tgt = s.forward(small_params(W, 4), traces=True, far_field=False)["traces"][0]
    s.set_target(tgt)
    return s


def test_alone_equals_mix_equals_batch(tomo):
    from tomography_gb300 import workloads as W

    A = _cands(W, 2, 111)
    B = _cands(W, 3, 222)
    C = _cands(W, 1, 333)
    with _solver(tomo, W) as s:
        batch = s.fitness_batch(A)
        ta = s.submit(A)
        alone = _drain(s, [ta], [2])[ta]
        # mix: B starts first, A joins while B runs, C joins later
        tb = s.submit(B)
        for _ in range(5):
            s.serve_step()
        ta2 = s.submit(A)
        for _ in range(3):
            s.serve_step()
        tc = s.submit(C)
        res = _drain(s, [tb, ta2, tc], [3, 2, 1])
        np.testing.assert_array_equal(alone, batch)
        np.testing.assert_array_equal(res[ta2], alone)
        np.testing.assert_array_equal(res[tb], s.fitness_batch(B))
        np.testing.assert_array_equal(res[tc], s.fitness_batch(C))


def test_mixed_grid_sizes_in_one_launch(tomo):
    from tomography_gb300 import workloads as W

    A = _cands(W, 2, 444)
    with _solver(tomo, W) as s:
        big = small_breast_spec(tomo, n_ellipses=4, steps=240, nx=128, ny=128)
        with tomo.Solver(big) as ref_solver:
            tgt = ref_solver.forward(small_params(W, 4), traces=True, far_field=False)["traces"][0]
            ref_solver.set_target(tgt)
            want_big = ref_solver.fitness_batch(A)
        s.set_target_for(big, tgt)
        want_small = s.fitness_batch(A)
        t1 = s.submit(A)
        t2 = s.submit(A, spec=big)
        res = _drain(s, [t1, t2], [2, 2])
        np.testing.assert_array_equal(res[t1], want_small)
        np.testing.assert_array_equal(res[t2], want_big)


def test_budget_admits_requests_as_memory_frees(tomo):
    """A budget of exactly one request's bytes: of three equal requests one is
    admitted, the other two wait in FIFO order, and each is admitted when the
    one before it retires and returns its memory (serve.cu admit()).  All three
    give the batch path's fitness bit for bit."""
    from tomography_gb300 import workloads as W

    A = _cands(W, 2, 555)
    with _solver(tomo, W) as s:
        want = s.fitness_batch(A)
        one = s.request_bytes(len(A))
        s.set_memory_budget(one)
        tickets = [s.submit(A) for _ in range(3)]
        s.serve_step()
        st = s.stats()
        assert st["serve_running"] == 1 and st["serve_queued"] == 2, st
        assert st["serve_running_solves"] == len(A) * s.n_exc
        assert st["serve_bytes_in_use"] == one
        done, order, seen_queued = {}, [], set()
        for _ in range(100000):
            n = s.serve_step()
            st = s.stats()
            assert st["serve_bytes_in_use"] <= one and st["serve_running"] <= 1, st
            seen_queued.add(st["serve_queued"])
            for t in tickets:
                if t not in done:
                    r = s.poll(t, len(A))
                    if r is not None:
                        done[t] = r
                        order.append(t)
            if len(done) == 3 and n == 0:
                break
        assert order == tickets                      # FIFO: admitted one after another
        assert {1, 0} <= seen_queued                 # the queue drained as memory freed up
        for t in tickets:
            np.testing.assert_array_equal(done[t], want)
        assert s.stats()["serve_bytes_in_use"] == 0


def test_budget_rejects_a_request_above_it(tomo):
    from tomography_gb300 import workloads as W

    A = _cands(W, 2, 556)
    with _solver(tomo, W) as s:
        s.set_memory_budget(s.request_bytes(len(A)) - 1)
        t = s.submit(A)
        with pytest.raises(tomo.TomoError) as ei:
            s.serve_step()
        assert ei.value.status == -2   # TOMO_ENOMEM_BUDGET: it can never fit
        with pytest.raises(tomo.TomoError) as ei:
            s.poll(t, 2)
        assert ei.value.status == -2
        with pytest.raises(tomo.TomoError):
            s.poll(t, 2)                # reported once, then forgotten
        s.set_memory_budget(0)
        t = s.submit(A)
        assert _drain(s, [t], [2])[t].shape == (2,)


def test_cancel(tomo):
    from tomography_gb300 import workloads as W

    A = _cands(W, 2, 557)
    with _solver(tomo, W) as s:
        want = s.fitness_batch(A)
        t1 = s.submit(A)
        t2 = s.submit(A)
        t3 = s.submit(A)
        s.serve_step()
        s.cancel(t2)
        res = _drain(s, [t1, t3], [2, 2])
        np.testing.assert_array_equal(res[t1], want)
        np.testing.assert_array_equal(res[t3], want)
        with pytest.raises(tomo.TomoError) as ei:
            s.poll(t2, 2)
        assert ei.value.status == -7   # TOMO_ECANCELLED
        with pytest.raises(tomo.TomoError) as ei:
            s.poll(t2, 2)              # reported once, then forgotten
        assert ei.value.status == -1


def test_bounded_wait(tomo):
    """tomo_wait: a zero timeout on a request nobody has stepped returns
    TOMO_ETIMEOUT and leaves the request queued; a generous one drives the loop
    to the batch path's bits."""
    from tomography_gb300 import workloads as W

    A = _cands(W, 2, 444)
    with _solver(tomo, W) as s:
        batch = s.fitness_batch(A)
        t = s.submit(A)
        with pytest.raises(tomo.TomoError) as ei:
            s.wait(t, 2, 0.0)
        assert ei.value.status == -3
        assert s.poll(t, 2) is None          # still queued
        got = s.wait(t, 2, 120.0)
        np.testing.assert_array_equal(got, batch)


def test_reference_mode_request_equals_batch(tomo):
    """A request in the reference GPU mode (plane waves, far-field misfit, the
    far field computed on the device for the misfit) gives the batch path's
    fitness bit for bit."""
    from tomography_gb300 import workloads as W

    spec = tomo.reference_spec(False).copy(steps=300)
    args = np.stack([W.reference_patch_args(900 + k) for k in range(2)])
    with tomo.Solver(spec) as s:
        target = s.forward(W.reference_patch_args(950), traces=False, far_field=True)["D"][0]
        s.set_target(target.ravel())
        batch = s.fitness_batch(args)
        t = s.submit(args)
        got = s.wait(t, 2, 120.0)
    np.testing.assert_array_equal(got, batch)
    assert np.all(batch < 0)
