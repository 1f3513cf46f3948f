"""Field snapshots of the last batch (tomo_field_snapshot).

* FP64 and FP32 final Ez, Hx, Hy of one transmitter solve against the FP64
  oracle's final fields: rel-L2 <= 1e-6 (FP64, rounded to float on export) and
  <= 1e-5 (FP32).
* The plain path and the batched path (which ends in the other ping-pong
  copy after an odd number of launches) give identical snapshots.
* Out-of-range requests are refused; a handle without a batch is not ready.
"""
from __future__ import annotations

import numpy as np
import pytest

from helpers import rel_l2, small_breast_spec, small_params

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec,tol", [("FP64", 1e-6), ("FP32", 1e-5)])
def test_snapshot_matches_oracle_fields(tomo, oracle, prec, tol):
    from tomography_gb300 import workloads as W

    spec = small_breast_spec(tomo, precision=getattr(tomo, prec), steps=301)
    params = small_params(W)
    with tomo.Solver(spec) as s:
        with pytest.raises(tomo.TomoError) as ei:
            s.field_snapshot()
        assert ei.value.status == -6   # TOMO_ENOTREADY
        s.forward(params, traces=False, far_field=False)
        got = {f: s.field_snapshot(0, 1, f) for f in ("ez", "hx", "hy")}
        with pytest.raises(tomo.TomoError):
            s.field_snapshot(1, 0, "ez")            # only one candidate in the batch
        with pytest.raises(tomo.TomoError):
            s.field_snapshot(0, spec.n_tx, "ez")    # excitation out of range
    ref = oracle.breast_forward(spec.as_dict(), params, txs=[1], fields=True)["problems"][0]
    for f in ("ez", "hx", "hy"):
        want = getattr(ref, f)
        assert got[f].shape == want.shape
        assert rel_l2(got[f], want) <= tol, (f, rel_l2(got[f], want))
    assert np.abs(got["ez"]).max() > 0


def test_plain_and_batched_snapshots_identical(tomo):
    from tomography_gb300 import workloads as W

    params = small_params(W)
    spec = small_breast_spec(tomo, steps=301, steps_per_launch=2, cols_per_lane=1)   # 151 launches: odd
    snaps = []
    for sp in (spec, spec.copy(plain=1)):
        with tomo.Solver(sp) as s:
            s.forward(params, traces=False, far_field=False)
            snaps.append([s.field_snapshot(0, 2, f) for f in ("ez", "hx", "hy")])
    for a, b in zip(*snaps):
        np.testing.assert_array_equal(a, b)
