"""Total-field variant of the reference GPU mode: the legacy far field of
oldFDTD_GPU.cu (H_inc_update :425-482, E_inc_update :655-717,
calculate_JandM_total :762-824), on the GPU against the FP64 oracle.

The oracle restates the legacy literally: one time loop advances the main grid
and then the incident vacuum grid, and one accumulator per contour point sums
H + H_inc and face-avg(Ez) + (face-avg(Ez_inc(n)) + face-avg(Ez_inc(n-1)))/2
with the M phasor at (n - 1/2) dt.  The product instead runs the incident grid
as one extra solve per batch, folds the two-level average into that solve's M
phasor and adds its sums in the far-field kernel.  These tests hold the
product's form to the literal one:

* FP64, 401x401, 600 steps, 4 plane waves: D rel-L2 <= 1e-6 (D leaves the
  device as float, 6e-8 relative rounding).
* FP32 at the legacy's full length (2000 steps): D rel-L2 <= 1e-4 and the
  absolute misfit against a target from another candidate, relative error
  <= 1e-4.
* The plain FP64 path (one solve per launch, the incident grid included)
  gives the batched path's D bit for bit.
* The serving loop refuses the variant (its batches carry no incident grid).
"""
from __future__ import annotations

import numpy as np
import pytest

from helpers import rel_l2

pytestmark = pytest.mark.gpu


def _spec(tomo, **kw):
    return tomo.reference_spec(False).copy(total_field=1, **kw)


def test_total_field_fp64_vs_oracle(tomo, oracle):
    from tomography_gb300 import workloads as W

    args = W.reference_patch_args(511)
    spec = _spec(tomo, precision=tomo.FP64, steps=600)
    with tomo.Solver(spec) as s:
        out = s.forward(args, traces=False, far_field=True)
    ref = oracle.reference_forward(spec.as_dict(), args)
    assert rel_l2(out["D"][0], ref["D"]) <= 1e-6
    # the variant changes the answer: without the incident grid and the
    # lagged M phasor the same candidate's far field differs by far more
    with tomo.Solver(spec.copy(total_field=0)) as s:
        scat = s.forward(args, traces=False, far_field=True)
    assert rel_l2(scat["D"][0], ref["D"]) > 1e-2


def test_total_field_fp32_full_length_vs_oracle(tomo, oracle):
    from tomography_gb300 import workloads as W

    args = W.reference_patch_args(512)
    other = W.reference_patch_args(513)
    spec = _spec(tomo)
    assert spec.steps == 2000
    ref = oracle.reference_forward(spec.as_dict(), args)
    target = oracle.reference_forward(spec.as_dict(), other)["D"].astype(np.float32)
    with tomo.Solver(spec) as s:
        s.set_target(target.ravel())
        out = s.forward(args, traces=False, far_field=True, fitness=True)
        st = s.stats()
    assert rel_l2(out["D"][0], ref["D"]) <= 1e-4
    want = oracle.misfit_abs(ref["D"].astype(np.float32), target, 4, 10)
    assert abs(out["fitness"][0] - want) <= 1e-4 * abs(want), (out["fitness"][0], want)
    # 4 excitations + the incident grid were advanced
    assert st["cell_updates"] == pytest.approx(5 * 401 * 401 * 2000)


def test_total_field_batch_equals_single_candidates(tomo):
    """Candidates of one batch share the batch's incident grid; each gets the
    same far field as when it runs alone."""
    from tomography_gb300 import workloads as W

    args = np.stack([W.reference_patch_args(520 + k) for k in range(3)])
    spec = _spec(tomo, steps=400, steps_per_launch=2, cols_per_lane=1)
    with tomo.Solver(spec) as s:
        batch = s.forward(args, traces=False, far_field=True)["D"]
        alone = [s.forward(args[k], traces=False, far_field=True)["D"][0] for k in range(3)]
    for k in range(3):
        np.testing.assert_array_equal(batch[k], alone[k])


def test_total_field_plain_bit_identical(tomo):
    from tomography_gb300 import workloads as W

    args = W.reference_patch_args(514)
    spec = _spec(tomo, precision=tomo.FP64, steps=300, steps_per_launch=1, cols_per_lane=1)
    with tomo.Solver(spec) as s:
        batched = s.forward(args, traces=False, far_field=True)
    with tomo.Solver(spec.copy(plain=1)) as s:
        plain = s.forward(args, traces=False, far_field=True)
    np.testing.assert_array_equal(plain["D"], batched["D"])
    assert np.abs(plain["D"]).max() > 0


def test_total_field_not_served(tomo):
    from tomography_gb300 import workloads as W

    spec = _spec(tomo, steps=100)
    with tomo.Solver(spec) as s:
        s.set_target(np.ones(4 * 10 * 100, dtype=np.float32))
        with pytest.raises(tomo.TomoError) as ei:
            s.submit(W.reference_patch_args(515))
        assert ei.value.status == -1
