"""The allocation-free trace misfit (tomo_trace_misfit_static), called through
the C ABI on device buffers the caller owns, against the fitness the
engine's own forward path computes from the same traces.

It serves callers that cannot allocate device memory themselves (their host
framework's allocator owns it, or their loop must not synchronise the device
through cudaMalloc/cudaFree); its scratch is a fixed device array shared by
every call, so the test also makes two calls in a row on the same buffers.
Tolerance: exact equality (the same reduction kernels run on the same
float traces).  This file is collected last on purpose.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from helpers import small_breast_spec, small_params

pytestmark = pytest.mark.gpu


def test_static_scratch_misfit_matches_forward(tomo):
    import torch

    from tomography_gb300 import workloads as W

    spec = small_breast_spec(tomo, n_ellipses=4, steps=240)
    cands = np.stack([W.candidate_params(777 + 1000 * k, 4, disc_radius=15e-3) for k in range(3)])
    with tomo.Solver(spec) as s:
        target = s.forward(small_params(W, 4), traces=True, far_field=False)["traces"][0]
        s.set_target(target)
        out = s.forward(cands, traces=True, far_field=False, fitness=True)
    n_cand, n_tx, n_rx, steps = out["traces"].shape
    dev = torch.device("cuda", 0)
    d_traces = torch.from_numpy(np.ascontiguousarray(out["traces"])).to(dev)
    d_target = torch.from_numpy(np.ascontiguousarray(target)).to(dev)
    d_fit = torch.full((n_cand,), float("nan"), dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    lib = tomo.library()
    for _ in range(2):   # two calls in a row share the static scratch
        d_fit.fill_(float("nan"))
        rc = lib.tomo_trace_misfit_static(C.c_void_p(d_traces.data_ptr()), C.c_void_p(d_target.data_ptr()), n_cand,
                                          n_tx, n_rx * steps, C.c_void_p(d_fit.data_ptr()), C.c_void_p(stream))
        assert rc == 0, lib.tomo_last_error()
        torch.cuda.synchronize(dev)
        np.testing.assert_array_equal(d_fit.cpu().numpy(), out["fitness"])
    # a non-finite trace value is not an error status here (the call stays
    # asynchronous): it shows up as a non-finite fitness of that candidate only
    bad = d_traces.clone()
    bad[1, 0, 0, 5] = float("nan")
    d_fit.fill_(0.0)
    rc = lib.tomo_trace_misfit_static(C.c_void_p(bad.data_ptr()), C.c_void_p(d_target.data_ptr()), n_cand, n_tx,
                                      n_rx * steps, C.c_void_p(d_fit.data_ptr()), C.c_void_p(stream))
    assert rc == 0, lib.tomo_last_error()
    torch.cuda.synchronize(dev)
    fit = d_fit.cpu().numpy()
    assert np.isnan(fit[1]) and fit[0] == out["fitness"][0] and fit[2] == out["fitness"][2]
    # sizes above the static limit are rejected before any launch
    rc = lib.tomo_trace_misfit_static(C.c_void_p(d_traces.data_ptr()), C.c_void_p(d_target.data_ptr()), 70000, 1,
                                      16, C.c_void_p(d_fit.data_ptr()), C.c_void_p(stream))
    assert rc == -1 and b"static scratch limit" in lib.tomo_last_error()
