"""Analytic known answers on the GPU.

Mirror symmetry: the Yee grid with its CPML is symmetric under y -> ny - y, so
with the transmitter on the symmetry row and a phantom symmetric about it, the
receivers k and N - k record the same trace.  Mirrored cells evaluate the same
explicitly rounded operations on the same values, so the traces are equal bit
for bit, in FP32 and FP64, at every blocking; and they match the FP64 oracle
(traces rel-L2 <= 1e-5 in FP32, <= 1e-10 in FP64).
"""
from __future__ import annotations

import numpy as np
import pytest

from helpers import rel_l2
from test_oracle import MIRROR_PARAMS, _mirror_spec, assert_doubled

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("blocking", [(0, 0), (4, 2), (2, 1)])
def test_mirror_symmetry(tomo, oracle, blocking):
    T, cols = blocking
    spec = _mirror_spec(tomo)
    ref = oracle.breast_forward(spec.as_dict(), MIRROR_PARAMS, bits=64)["traces"][0]
    for prec, tol in ((tomo.FP32, 1e-5), (tomo.FP64, 1e-10)):
        c = cols if prec == tomo.FP32 else min(cols, 1)
        with tomo.Solver(spec.copy(precision=prec, steps_per_launch=T, cols_per_lane=c)) as s:
            tr = s.forward(MIRROR_PARAMS, traces=True, traces_f64=True, far_field=False)["traces_f64"][0][0]
        for k in range(1, 8):
            np.testing.assert_array_equal(tr[k], tr[16 - k])
        assert rel_l2(tr, ref) <= tol, prec


def test_source_linearity_exact(tomo):
    """Twice the source amplitude gives exactly twice every trace: in FP64
    everywhere, in FP32 wherever |2a| >= 1e-30 (the arrival's leading edge
    passes through subnormal values, where doubling and rounding do not
    commute; those differences stay below 1.2e-38)."""
    spec = _mirror_spec(tomo)
    for prec in (tomo.FP32, tomo.FP64):
        out = {}
        for amp in (1.0e3, 2.0e3):
            with tomo.Solver(spec.copy(precision=prec, src_amp=amp)) as s:
                out[amp] = s.forward(MIRROR_PARAMS, traces=True, traces_f64=True, far_field=False)["traces_f64"][0]
        assert_doubled(out[2.0e3], out[1.0e3], 64 if prec == tomo.FP64 else 32)


def test_reciprocity(tomo):
    """The GPU solves keep the scheme's reciprocity: trace(tx a, rx b) equals
    trace(tx b, rx a) for every antenna pair, to rel-L2 <= 1e-12 in FP64 and
    <= 1e-5 in FP32."""
    from tomography_gb300 import workloads as W

    from helpers import small_params
    from test_oracle import _reciprocity_spec, reciprocity_error

    spec = _reciprocity_spec(tomo)
    params = small_params(W, 3)
    for prec, tol in ((tomo.FP64, 1e-12), (tomo.FP32, 1e-5)):
        with tomo.Solver(spec.copy(precision=prec)) as s:
            tr = s.forward(params, traces=True, traces_f64=True, far_field=False)["traces_f64"][0]
        assert reciprocity_error(tr) <= tol, prec
