"""GPU parity: the CUDA path through the C ABI against the CPU oracle.

Tolerances (stated per check):
* FP64 GPU vs FP64 oracle: receiver traces rel-L2 <= 1e-10 (same formulas; only
  FMA contraction and reciprocal-vs-divide rounding differ).
* FP32 GPU vs FP64 oracle: receiver-trace rel-L2 <= 1e-5 and fitness relative
  error <= 1e-6 (the target stated for the FP32 path).
* Temporal-blocking depths and columns-per-lane: bit-identical traces (every
  cell performs the same operations whatever the blocking).
"""
from __future__ import annotations

import numpy as np
import pytest

from helpers import rel_l2, small_breast_spec, small_params

pytestmark = pytest.mark.gpu


def _oracle_traces(oracle, spec, params, bits=64):
    return oracle.breast_forward(spec.as_dict(), params, bits=bits)


def test_breast_fp64_matches_oracle(tomo, oracle):
    from tomography_gb300 import workloads as W

    spec = small_breast_spec(tomo, precision=tomo.FP64, steps_per_launch=1, cols_per_lane=1)
    params = small_params(W)
    with tomo.Solver(spec) as s:
        out = s.forward(params, traces=True, traces_f64=True, far_field=True)
    ref = _oracle_traces(oracle, spec, params)
    err = rel_l2(out["traces_f64"][0], ref["traces"])
    assert err <= 1e-10, err
    # far field (float output of an FP64 transform)
    errD = rel_l2(out["D"][0], ref["D"])
    assert errD <= 1e-5, errD


def test_breast_fp32_matches_fp64_oracle(tomo, oracle):
    from tomography_gb300 import workloads as W

    spec = small_breast_spec(tomo)
    params = small_params(W)
    with tomo.Solver(spec) as s:
        out = s.forward(params, traces=True, far_field=True)
    ref = _oracle_traces(oracle, spec, params)
    err = rel_l2(out["traces"][0], ref["traces"])
    assert err <= 1e-5, err
    errD = rel_l2(out["D"][0], ref["D"])
    assert errD <= 1e-4, errD


@pytest.mark.parametrize("T_cols", [(1, 1), (2, 1), (2, 2), (2, 4), (3, 1), (3, 2), (4, 1), (4, 2), (6, 1), (8, 1)])
def test_blocking_depths_bit_identical(tomo, T_cols):
    from tomography_gb300 import workloads as W

    T, cols = T_cols
    params = small_params(W)
    base = small_breast_spec(tomo, steps=203, steps_per_launch=1, cols_per_lane=1)
    with tomo.Solver(base) as s:
        ref = s.forward(params, traces=True, far_field=True)
    spec = small_breast_spec(tomo, steps=203, steps_per_launch=T, cols_per_lane=cols)
    with tomo.Solver(spec) as s:
        out = s.forward(params, traces=True, far_field=True)
    np.testing.assert_array_equal(out["traces"], ref["traces"])
    np.testing.assert_array_equal(out["D"], ref["D"])


@pytest.mark.parametrize("T_cols", [(2, 1), (2, 2), (2, 4), (3, 1), (3, 2), (4, 1), (4, 2)])
def test_wide_and_narrow_items_bit_identical(tomo, T_cols):
    """A 200x200 grid, where COLS = 2 blockings split each solve into narrow
    edge strips and wide interior strips (the 96x96 grid above is narrow
    throughout): the same bits as one step per launch, one column per lane."""
    from tomography_gb300 import workloads as W

    T, cols = T_cols
    base = tomo.breast_spec(0).copy(steps=301, n_tx=2)
    params = W.phantom_params(W.config_seed(0) + 3, base.n_ellipses)
    with tomo.Solver(base.copy(steps_per_launch=1, cols_per_lane=1)) as s:
        ref = s.forward(params, traces=True, far_field=True)
    with tomo.Solver(base.copy(steps_per_launch=T, cols_per_lane=cols)) as s:
        out = s.forward(params, traces=True, far_field=True)
    np.testing.assert_array_equal(out["traces"], ref["traces"])
    np.testing.assert_array_equal(out["D"], ref["D"])
    assert np.abs(ref["traces"]).max() > 0


@pytest.mark.parametrize("blocking", [(4, 2, 2), (3, 2, 2), (2, 4, 2), (2, 2, 3), (2, 2, 2)])
def test_every_wide_variant_bit_identical(tomo, blocking, monkeypatch):
    """Each compiled wide variant (T, COLS, minimum resident blocks per SM,
    fixed through TOMO_T / TOMO_COLS / TOMO_MINB) on the 200x200 grid, which
    has narrow edge strips and wide interior strips: the bits of one step
    per launch, one column per lane."""
    from tomography_gb300 import workloads as W

    T, cols, minb = blocking
    base = tomo.breast_spec(0).copy(steps=301, n_tx=2)
    params = W.phantom_params(W.config_seed(0) + 5, base.n_ellipses)
    with tomo.Solver(base.copy(steps_per_launch=1, cols_per_lane=1)) as s:
        ref = s.forward(params, traces=True, far_field=True)
    monkeypatch.setenv("TOMO_T", str(T))
    monkeypatch.setenv("TOMO_COLS", str(cols))
    monkeypatch.setenv("TOMO_MINB", str(minb))
    with tomo.Solver(base) as s:
        out = s.forward(params, traces=True, far_field=True)
        st = s.stats()
    assert (st["steps_per_launch"], st["cols_per_lane"], st["min_blocks_per_sm"]) == blocking
    np.testing.assert_array_equal(out["traces"], ref["traces"])
    np.testing.assert_array_equal(out["D"], ref["D"])


@pytest.mark.parametrize("nseg", [5, 13])
def test_row_segments_bit_identical(tomo, nseg, monkeypatch):
    """Strips cut into row segments (used when a batch is too small to fill
    the GPU; each segment recomputes 2T halo rows) give the same bits as whole
    strips: fields, receiver traces and far field."""
    from tomography_gb300 import workloads as W

    spec = tomo.breast_spec(0).copy(steps=301, n_tx=2, steps_per_launch=2, cols_per_lane=2)
    params = W.phantom_params(W.config_seed(0) + 5, spec.n_ellipses)
    monkeypatch.setenv("TOMO_SEGMENTS", "1")
    with tomo.Solver(spec) as s:
        ref = s.forward(params, traces=True, far_field=True)
    monkeypatch.setenv("TOMO_SEGMENTS", str(nseg))
    with tomo.Solver(spec) as s:
        out = s.forward(params, traces=True, far_field=True)
    np.testing.assert_array_equal(out["traces"], ref["traces"])
    np.testing.assert_array_equal(out["D"], ref["D"])


def test_fitness_fp32_vs_oracle(tomo, oracle):
    from tomography_gb300 import workloads as W

    spec = small_breast_spec(tomo, n_ellipses=4)
    target_params = small_params(W, n_ellipses=4, seed_offset=1)
    cand = small_params(W, n_ellipses=4, seed_offset=7)
    tgt = _oracle_traces(oracle, spec, target_params)["traces"]
    with tomo.Solver(spec) as s:
        s.set_target(tgt.astype(np.float32))
        fit = s.fitness(cand)
    got = _oracle_traces(oracle, spec, cand)["traces"]
    want = oracle.misfit_trace(got, tgt.astype(np.float32))
    assert abs(fit - want) <= 1e-6 * abs(want), (fit, want)


def test_fitness_batch_equals_single(tomo):
    from tomography_gb300 import workloads as W

    spec = small_breast_spec(tomo, n_ellipses=4)
    cands = np.stack([W.candidate_params(1234 + 1000 * k, 4, disc_radius=15e-3) for k in range(5)])
    with tomo.Solver(spec) as s:
        tgt = s.forward(small_params(W, 4), traces=True, far_field=False)["traces"][0]
        s.set_target(tgt)
        batch = s.fitness_batch(cands)
        singles = np.array([s.fitness(c) for c in cands])
    np.testing.assert_array_equal(batch, singles)
    assert np.all(batch < 0)


def test_reference_gpu_mode_matches_oracle(tomo, oracle):
    """FDTD_GPU semantics (3x3 Debye patches, centred plane wave, NaN clamp) on the
    reference's own 401x401 grid, 400 of its 2000 steps, all 4 excitations."""
    from tomography_gb300 import workloads as W

    args = W.reference_patch_args(99)
    for prec, tolD in ((tomo.FP64, 1e-5), (tomo.FP32, 2e-4)):
        spec = tomo.reference_spec(False).copy(steps=400, precision=prec)
        with tomo.Solver(spec) as s:
            out = s.forward(args, traces=False, far_field=True)
        ref = oracle.reference_forward(spec.as_dict(), args)
        err = rel_l2(out["D"][0], ref["D"])
        assert err <= tolD, (prec, err)
