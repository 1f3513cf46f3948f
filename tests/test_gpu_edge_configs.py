"""Grid and boundary configurations off the workloads' beaten path, on the GPU
against the FP64 oracle (breast-imaging mode, one seeded phantom, 3
transmitters):

* a non-square grid (150 x 90): strips, row segments and the contour of an
  nx != ny grid;
* no CPML (ncpml = 0: PEC walls right at the boundary), contour 4 cells in;
* the widest CPML the engine takes (32 cells on a 160 x 160 grid);
* no near-to-far-field transform (nfreq = 0): traces only.

Each at the autotuned blocking and at T = 4 (two columns per lane in FP32;
FP64 is compiled with one).
Tolerances: FP32 traces rel-L2 <= 1e-5, FP64 traces <= 1e-10, far field D
rel-L2 <= 1e-4 (FP32) and <= 1e-6 (FP64; D leaves the device as float).
"""
from __future__ import annotations

import numpy as np
import pytest

from helpers import rel_l2, small_params

pytestmark = pytest.mark.gpu

CASES = {
    "non_square": dict(nx=150, ny=90, ncpml=8, nf2ff_d=11, disc_radius=12e-3, antenna_radius=15e-3),
    "no_cpml": dict(nx=96, ny=96, ncpml=0, nf2ff_d=4, disc_radius=15e-3, antenna_radius=19e-3),
    "wide_cpml": dict(nx=160, ny=160, ncpml=32, nf2ff_d=35, disc_radius=15e-3, antenna_radius=19e-3),
    "no_ntff": dict(nx=96, ny=96, ncpml=8, nf2ff_d=11, nfreq=0, disc_radius=15e-3, antenna_radius=19e-3),
}


def _spec(tomo, case, **kw):
    base = dict(steps=300, n_antennas=8, n_tx=3, n_angles=36, n_ellipses=3)
    base.update(CASES[case])
    base.update(kw)
    return tomo.breast_spec(0).copy(**base)


@pytest.mark.parametrize("blocking", [(0, 0), (4, 2)])
@pytest.mark.parametrize("case", sorted(CASES))
def test_configuration_vs_oracle(tomo, oracle, case, blocking):
    from tomography_gb300 import workloads as W

    T, cols = blocking
    spec = _spec(tomo, case)
    params = small_params(W, 3)
    if case == "non_square":
        params = W.phantom_params(W.config_seed(0) + 1, 3, disc_radius=12e-3)
    ref = oracle.breast_forward(spec.as_dict(), params, bits=64)
    for prec, tr_tol, d_tol in ((tomo.FP32, 1e-5, 1e-4), (tomo.FP64, 1e-10, 1e-6)):
        c = cols if prec == tomo.FP32 else min(cols, 1)
        with tomo.Solver(spec.copy(precision=prec, steps_per_launch=T, cols_per_lane=c)) as s:
            out = s.forward(params, traces=True, traces_f64=True, far_field=spec.nfreq > 0)
        assert rel_l2(out["traces_f64"][0], ref["traces"]) <= tr_tol, (case, prec)
        if spec.nfreq > 0:
            assert rel_l2(out["D"][0], ref["D"]) <= d_tol, (case, prec)
    assert np.abs(ref["traces"]).max() > 0
