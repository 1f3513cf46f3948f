"""Precision study at the size of the breast-imaging precision workload.

One seeded phantom on a 600x600 grid (dx = 0.25 mm, 6000 steps, 32 antennas
at 70 mm, all transmitting; NTFF at 8 frequencies, 360 angles), solved three
ways: FP32 fields with Kahan-compensated FP32 DFT sums, FP64 fields with FP64
sums (both on the GPU), and the FP64 CPU oracle.

Tolerances:
* FP64 GPU vs FP64 oracle: receiver traces rel-L2 <= 1e-10, far field <= 1e-6.
* FP32 GPU vs FP64 oracle: all receiver traces together rel-L2 <= 1e-5; every
  (transmitter, receiver) trace rel-L2 <= 1e-4; far field rel-L2 <= 1e-4;
  fitness (trace misfit against a second seeded phantom) relative error <= 1e-6.
The measured errors are printed as one JSON line (run pytest with -s).
"""
from __future__ import annotations

import json

import numpy as np
import pytest

from helpers import rel_l2

pytestmark = pytest.mark.gpu


def test_precision_study_600(tomo, oracle):
    from tomography_gb300 import workloads as W

    spec = tomo.breast_spec(2)
    params = W.phantom_params(W.config_seed(2), spec.n_ellipses)
    target_params = W.phantom_params(W.config_seed(2) + 1, spec.n_ellipses)
    out = {}
    for name, prec in (("fp32", tomo.FP32), ("fp64", tomo.FP64)):
        with tomo.Solver(spec.copy(precision=prec)) as s:
            o = s.forward(params, traces=True, traces_f64=True, far_field=True)
            t = s.forward(target_params, traces=True, traces_f64=True, far_field=False)
        out[name] = (o["traces_f64"][0], o["D"][0], t["traces_f64"][0])
    ref = oracle.breast_forward(spec.as_dict(), params, bits=64)
    tr_ref, D_ref = ref["traces"], ref["D"]
    target = out["fp64"][2].astype(np.float32)

    def per_rx(tr):
        num = np.linalg.norm((tr - tr_ref).reshape(tr_ref.shape[0], tr_ref.shape[1], -1), axis=2)
        den = np.linalg.norm(tr_ref.reshape(tr_ref.shape[0], tr_ref.shape[1], -1), axis=2)
        return num / den

    fit_ref = oracle.misfit_trace(tr_ref.astype(np.float32), target)
    report = {}
    for name in ("fp32", "fp64"):
        tr, D, _ = out[name]
        pr = per_rx(tr)
        fit = oracle.misfit_trace(tr.astype(np.float32), target)
        report[name] = {"trace_rel_l2": rel_l2(tr, tr_ref), "per_receiver_max": float(pr.max()),
                        "per_receiver_median": float(np.median(pr)), "far_field_rel_l2": rel_l2(D, D_ref),
                        "fitness": fit, "fitness_rel_err": abs(fit - fit_ref) / abs(fit_ref)}
    report["oracle_fitness"] = fit_ref
    print(json.dumps({"precision_study_600": report}))
    r64, r32 = report["fp64"], report["fp32"]
    assert r64["trace_rel_l2"] <= 1e-10 and r64["far_field_rel_l2"] <= 1e-6, r64
    assert r32["trace_rel_l2"] <= 1e-5, r32
    assert r32["per_receiver_max"] <= 1e-4, r32
    assert r32["far_field_rel_l2"] <= 1e-4, r32
    assert r32["fitness_rel_err"] <= 1e-6, r32
