"""Large-batch workload (breast workload 4: 2048x2048, dx 0.125 mm, 16-cell
CPML, 20000 steps, 32 transmitters, 16 ellipses in a skin-layer disc, NTFF at
16 frequencies over 720 angles) on the GPU, one seeded candidate.

* Against the FP64 oracle at a reduced step count (1200 steps, 5 G
  cell-updates per solve, about a minute of host time for two solves), the
  first two transmitters: FP32 receiver traces rel-L2 <= 1e-5 and far field D
  rel-L2 <= 1e-4; FP64 traces rel-L2 <= 1e-10.  By step 1200 the pulse
  (centred at step 195) has crossed the phantom disc and reached the
  neighbouring antennas.
* At the full 20000 steps, where the oracle would take hours, FP32 against
  the FP64 GPU path on the same two transmitters: traces rel-L2 <= 1e-5, far
  field rel-L2 <= 1e-4.  The FP64 GPU path is itself held to the oracle by the
  reduced-step check above and the precision study.
* The full-size state of a 64-candidate batch (about 340 GB) exceeds one GPU;
  the batch path rejects it against a memory budget instead of failing in
  cudaMalloc.
"""
from __future__ import annotations

import numpy as np
import pytest

from helpers import rel_l2

pytestmark = pytest.mark.gpu


def _candidate(W, spec):
    return W.candidate_batch(4, 1, spec.n_ellipses, disc_radius=spec.disc_radius)


def test_large_reduced_steps_vs_oracle(tomo, oracle):
    from tomography_gb300 import workloads as W

    spec = tomo.breast_spec(4).copy(steps=1200, n_tx=2)
    cand = _candidate(W, spec)
    ref = oracle.breast_forward(spec.as_dict(), cand[0], bits=64)
    for prec, tr_tol in ((tomo.FP32, 1e-5), (tomo.FP64, 1e-10)):
        with tomo.Solver(spec.copy(precision=prec)) as s:
            out = s.forward(cand, traces=True, traces_f64=True, far_field=True)
        assert rel_l2(out["traces_f64"][0], ref["traces"]) <= tr_tol, prec
        assert rel_l2(out["D"][0], ref["D"]) <= 1e-4, prec
    # the pulse reached more than the transmitting antenna
    tr = ref["traces"][0]
    assert (np.abs(tr).max(axis=1) > 1e-3 * np.abs(tr).max()).sum() >= 3


def test_large_full_steps_fp32_vs_fp64(tomo):
    from tomography_gb300 import workloads as W

    spec = tomo.breast_spec(4).copy(n_tx=2)
    assert spec.steps == 20000 and spec.nx == 2048
    cand = _candidate(W, spec)
    res = {}
    for name, prec in (("fp32", tomo.FP32), ("fp64", tomo.FP64)):
        with tomo.Solver(spec.copy(precision=prec)) as s:
            res[name] = s.forward(cand, traces=True, traces_f64=True, far_field=True)
    t32, t64 = res["fp32"]["traces_f64"][0], res["fp64"]["traces_f64"][0]
    assert rel_l2(t32, t64) <= 1e-5
    assert rel_l2(res["fp32"]["D"][0], res["fp64"]["D"][0]) <= 1e-4


def test_large_full_batch_is_refused_by_budget(tomo):
    from tomography_gb300 import workloads as W

    spec = tomo.breast_spec(4)
    with tomo.Solver(spec) as s:
        need = s.request_bytes(64)
        assert need > 250e9
        s.set_memory_budget(int(200e9))
        with pytest.raises(tomo.TomoError) as ei:
            s.forward(W.candidate_batch(4, 64, spec.n_ellipses, disc_radius=spec.disc_radius), traces=False,
                      far_field=False)
        assert ei.value.status == -2
