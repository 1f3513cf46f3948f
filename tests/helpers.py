"""Shared test helpers: small problem specs and error metrics."""
from __future__ import annotations

import numpy as np


def rel_l2(got, want) -> float:
    """Relative L2 error; complex arrays (DFT surface currents) compare both parts."""
    got, want = np.asarray(got), np.asarray(want)
    dt = np.complex128 if (np.iscomplexobj(got) or np.iscomplexobj(want)) else np.float64
    got = got.astype(dt)
    want = want.astype(dt)
    den = np.linalg.norm(want)
    return float(np.linalg.norm(got - want) / den) if den > 0 else float(np.linalg.norm(got))


def small_breast_spec(T, **kw):
    """A 96x96 breast-mode problem that the oracle finishes in about a second:
    same physics and CPML/source parameterisation as workload 0, smaller disc
    and antenna ring."""
    base = dict(nx=96, ny=96, steps=300, ncpml=8, nf2ff_d=11, disc_radius=15e-3, antenna_radius=19e-3,
                n_antennas=8, n_tx=3, n_angles=36, n_ellipses=3)
    base.update(kw)
    return T.breast_spec(0).copy(**base)


def small_params(W, n_ellipses=3, seed_offset=1):
    return W.phantom_params(W.config_seed(0) + seed_offset, n_ellipses, disc_radius=15e-3)
