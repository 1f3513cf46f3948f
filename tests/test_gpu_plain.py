"""The plain one-solve-per-launch path and the (T, COLS) autotuner.

* Plain path (H, E and DFT kernels per step, one solve per launch) against the
  wavefront path: bit-identical traces, far field and fitness, in FP64 and
  FP32, in the breast-imaging and the reference modes -- both evaluate the same
  explicitly rounded formulas in the same order.
* Plain FP64 against the FP64 oracle: receiver traces rel-L2 <= 1e-10.
* Autotuner (steps_per_launch = cols_per_lane = 0): times several pairs on the
  first batch of a size, caches the choice for the next batch of that size,
  and gives the same bits as a fixed pair.
"""
from __future__ import annotations

import numpy as np
import pytest

from helpers import rel_l2, small_breast_spec, small_params

pytestmark = pytest.mark.gpu


def _forward(tomo, spec, params, **kw):
    with tomo.Solver(spec) as s:
        out = s.forward(params, **kw)
        st = s.stats()
    return out, st


@pytest.mark.parametrize("prec", ["FP64", "FP32"])
def test_plain_breast_bit_identical_to_wavefront(tomo, prec):
    from tomography_gb300 import workloads as W

    params = small_params(W)
    spec = small_breast_spec(tomo, precision=getattr(tomo, prec), steps=257, steps_per_launch=2, cols_per_lane=1)
    batched, _ = _forward(tomo, spec, params, traces=True, far_field=True)
    plain, st = _forward(tomo, spec.copy(plain=1), params, traces=True, far_field=True)
    np.testing.assert_array_equal(plain["traces"], batched["traces"])
    np.testing.assert_array_equal(plain["D"], batched["D"])
    # one solve per launch: 3 kernels (H, E, DFT) per step and solve
    assert st["kernels"] >= 3 * spec.steps * spec.n_tx


def test_plain_fp64_matches_oracle(tomo, oracle):
    from tomography_gb300 import workloads as W

    spec = small_breast_spec(tomo, precision=tomo.FP64, plain=1)
    params = small_params(W)
    out, _ = _forward(tomo, spec, params, traces=True, traces_f64=True, far_field=True)
    ref = oracle.breast_forward(spec.as_dict(), params, bits=64)
    assert rel_l2(out["traces_f64"][0], ref["traces"]) <= 1e-10
    assert rel_l2(out["D"][0], ref["D"]) <= 1e-5


@pytest.mark.parametrize("prec", ["FP64", "FP32"])
def test_plain_reference_mode_bit_identical(tomo, prec):
    """FDTD_GPU semantics (plane waves, Debye patches, NaN clamp) on a reduced
    step count of the reference's own 401x401 grid."""
    from tomography_gb300 import workloads as W

    args = W.reference_patch_args(31)
    spec = tomo.reference_spec(False).copy(steps=300, precision=getattr(tomo, prec), steps_per_launch=1,
                                           cols_per_lane=1)
    batched, _ = _forward(tomo, spec, args, traces=False, far_field=True)
    plain, _ = _forward(tomo, spec.copy(plain=1), args, traces=False, far_field=True)
    np.testing.assert_array_equal(plain["D"], batched["D"])
    assert np.abs(plain["D"]).max() > 0


def test_autotuner_caches_and_matches_fixed_blocking(tomo):
    from tomography_gb300 import workloads as W

    spec = small_breast_spec(tomo, n_ellipses=4, steps=400)
    cands = np.stack([W.candidate_params(777 + 1000 * k, 4, disc_radius=15e-3) for k in range(3)])
    fixed, _ = _forward(tomo, spec.copy(steps_per_launch=1, cols_per_lane=1), cands, traces=True, far_field=True)
    with tomo.Solver(spec.copy(steps_per_launch=0, cols_per_lane=0)) as s:
        first = s.forward(cands, traces=True, far_field=True)
        st1 = s.stats()
        second = s.forward(cands, traces=True, far_field=True)
        st2 = s.stats()
        single = s.forward(cands[:1], traces=True, far_field=True)
        st3 = s.stats()
    assert st1["tuned_configs"] >= 2 and st1["tune_ms"] > 0
    assert st2["tuned_configs"] == 0 and st2["tune_ms"] == 0        # cached for this batch size
    assert st3["tuned_configs"] >= 2                                # a new batch size is tuned again
    assert (st2["steps_per_launch"], st2["cols_per_lane"]) == (st1["steps_per_launch"], st1["cols_per_lane"])
    for out in (first, second):
        np.testing.assert_array_equal(out["traces"], fixed["traces"])
        np.testing.assert_array_equal(out["D"], fixed["D"])
    np.testing.assert_array_equal(single["traces"][0], fixed["traces"][0])


def test_autotuner_respects_fixed_dimension(tomo):
    from tomography_gb300 import workloads as W

    spec = small_breast_spec(tomo, steps=400, steps_per_launch=0, cols_per_lane=1)
    with tomo.Solver(spec) as s:
        s.forward(small_params(W), traces=False, far_field=False)
        st = s.stats()
    assert st["cols_per_lane"] == 1
    assert st["tuned_configs"] >= 2
