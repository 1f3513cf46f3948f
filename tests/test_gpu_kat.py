"""Analytic known answers on the GPU.

Mirror symmetry: the Yee grid with its CPML is symmetric under y -> ny - y, so
with the transmitter on the symmetry row and a phantom symmetric about it, the
receivers k and N - k record the same trace.  Mirrored cells evaluate the same
explicitly rounded operations on the same values, so the traces are equal bit
for bit, in FP32 and FP64, at every blocking; and they match the FP64 oracle
(traces rel-L2 <= 1e-5 in FP32, <= 1e-10 in FP64).  Source linearity and
reciprocity hold as in the oracle.  In a homogeneous background the GPU's
pulse travels at c0 / sqrt(eps_r) with 1/sqrt(r) spreading, and its CPML
reflects as little as the oracle's.
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


BACKGROUND_ELLIPSE = np.array([0.0, 0.0, 3e-3, 3e-3, 0.0, 9.0, 1e-9, 0.0])   # delta_eps 1e-9: the usual Jp box


def _homogeneous_gpu_spec(tomo, n, ncpml, steps, radius, precision):
    """The homogeneous background through the GPU's ordinary paths: the disc
    and one ellipse (BACKGROUND_ELLIPSE) made of the background material.  The
    ellipse keeps a delta_eps of 1e-9, so that the dispersive (Jp) box is not
    empty, as in every phantom; its effect on the traces is of that order."""
    return tomo.breast_spec(0).copy(nx=n, ny=n, steps=steps, ncpml=ncpml, disc_radius=10e-3, disc_eps_inf=9.0,
                                    disc_del_eps=0.0, disc_sigma=0.0, n_ellipses=1, n_antennas=16, n_tx=1,
                                    antenna_radius=radius, nfreq=0, precision=precision)


def _traces(tomo, spec):
    with tomo.Solver(spec) as s:
        return s.forward(BACKGROUND_ELLIPSE, traces=True, traces_f64=True, far_field=False)["traces_f64"][0][0]


def test_free_space_propagation(tomo, oracle):
    """The GPU's traces in the homogeneous background match the FP64 oracle
    (rel-L2 <= 1e-5 in FP32, <= 1e-10 in FP64) and obey the free-space known
    answer: envelope-peak delay slope within 2 % of sqrt(eps_r)/c0, intercept
    within 5 dt of the source peak, amplitude x sqrt(r) constant to 1 %."""
    pytest.importorskip("scipy.signal")
    from test_oracle import free_space_fit

    for prec, tol in ((tomo.FP32, 1e-5), (tomo.FP64, 1e-10)):
        spec = _homogeneous_gpu_spec(tomo, 200, 10, 1400, 30e-3, prec)
        tr = _traces(tomo, spec)
        d = spec.as_dict()
        assert rel_l2(tr, oracle.breast_forward(d, BACKGROUND_ELLIPSE, bits=64)["traces"][0]) <= tol, prec
        slope_v, t0_steps, spread = free_space_fit(tr, d, oracle)
        assert abs(slope_v - 1.0) < 0.02 and abs(t0_steps) < 5 and spread < 0.01, prec


def test_cpml_reflection(tomo):
    """The GPU's CPML absorbs as the oracle's does: the traces of a 140x140
    grid (10-cell CPML) and of a 420x420 grid whose boundary is out of reach
    differ by less than 1e-4 of the direct signal (oracle: 3.6e-6), in FP32
    and FP64; PEC walls (no CPML) send back more than 5 % in the same window."""
    for prec in (tomo.FP32, tomo.FP64):
        big = _traces(tomo, _homogeneous_gpu_spec(tomo, 420, 10, 1500, 25e-3, prec))
        ref = np.abs(big).max()
        r10 = np.abs(_traces(tomo, _homogeneous_gpu_spec(tomo, 140, 10, 1500, 25e-3, prec)) - big).max() / ref
        pec = np.abs(_traces(tomo, _homogeneous_gpu_spec(tomo, 140, 0, 1500, 25e-3, prec)) - big).max() / ref
        assert r10 < 1e-4 and pec > 0.05, (prec, r10, pec)
