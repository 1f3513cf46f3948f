"""Seeded synthetic workloads of the breast-imaging configurations.

One project-owned generator (splitmix64 -> uniform double in [0, 1)) so that
every run, on any host, draws the same phantoms and candidates.  Seed of
workload ``config`` is ``0x70F00000 + config``; candidate ``k`` uses
``seed + 1000*k``; the target phantom uses ``seed + 1``.

Parameter vector of one candidate: 8 values per ellipse,
``(cx, cy, a, b, angle, eps_inf, del_eps, sigma)`` in metres / radians / S/m.
"""
from __future__ import annotations

import math

import numpy as np

MASK64 = (1 << 64) - 1
FAT = (3.1, 1.6, 0.036)
FIBRO = (12.9, 24.6, 0.397)


class SplitMix64:
    def __init__(self, seed: int):
        self.state = seed & MASK64

    def next_u64(self) -> int:
        self.state = (self.state + 0x9E3779B97F4A7C15) & MASK64
        z = self.state
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & MASK64
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & MASK64
        return z ^ (z >> 31)

    def uniform(self) -> float:
        return (self.next_u64() >> 11) * (1.0 / (1 << 53))


def config_seed(config: int) -> int:
    return 0x70F00000 + config


def _ellipse_centre(rng: SplitMix64, disc_radius: float) -> tuple[float, float]:
    r = disc_radius * math.sqrt(rng.uniform())
    phi = 2 * math.pi * rng.uniform()
    return r * math.cos(phi), r * math.sin(phi)


def phantom_params(seed: int, n_ellipses: int, disc_radius: float = 35e-3,
                   axes=(3e-3, 10e-3), material=FIBRO) -> np.ndarray:
    """Target phantom: n fibroglandular ellipses inside the fat disc."""
    rng = SplitMix64(seed)
    out = []
    for _ in range(n_ellipses):
        cx, cy = _ellipse_centre(rng, disc_radius)
        a = axes[0] + (axes[1] - axes[0]) * rng.uniform()
        b = axes[0] + (axes[1] - axes[0]) * rng.uniform()
        ang = math.pi * rng.uniform()
        out += [cx, cy, a, b, ang, material[0], material[1], material[2]]
    return np.array(out, dtype=np.float64)


def candidate_params(seed: int, n_ellipses: int, disc_radius: float = 35e-3) -> np.ndarray:
    """One PSO candidate drawn uniformly within the per-parameter bounds."""
    rng = SplitMix64(seed)
    out = []
    for _ in range(n_ellipses):
        cx, cy = _ellipse_centre(rng, disc_radius)
        a = 2e-3 + 13e-3 * rng.uniform()
        b = 2e-3 + 13e-3 * rng.uniform()
        ang = math.pi * rng.uniform()
        einf = 2 + 18 * rng.uniform()
        deps = 1 + 39 * rng.uniform()
        sig = rng.uniform()
        out += [cx, cy, a, b, ang, einf, deps, sig]
    return np.array(out, dtype=np.float64)


def candidate_batch(config: int, n_cand: int, n_ellipses: int, disc_radius: float = 35e-3) -> np.ndarray:
    seed = config_seed(config)
    return np.stack([candidate_params(seed + 1000 * k, n_ellipses, disc_radius) for k in range(n_cand)])


def target_phantom(config: int, n_ellipses: int = 3, disc_radius: float = 35e-3) -> np.ndarray:
    return phantom_params(config_seed(config) + 1, n_ellipses, disc_radius)


def reference_patch_args(seed: int, cpu_variant: bool = False) -> np.ndarray:
    """Random reference-mode arguments within the reference's search bounds
    (test.cxx:60-77: eps_inf in [1, 7], del_eps in [1.5, 41]; sigma in [0, 0.1])."""
    rng = SplitMix64(seed)
    if cpu_variant:
        eps = [1 + 9 * rng.uniform() for _ in range(81)]
        sig = [0.1 * rng.uniform() for _ in range(81)]
        return np.array(eps + sig, dtype=np.float64)
    einf = [1 + 6 * rng.uniform() for _ in range(9)]
    deps = [1.5 + 39.5 * rng.uniform() for _ in range(9)]
    sig = [0.1 * rng.uniform() for _ in range(9)]
    return np.array(einf + deps + sig, dtype=np.float64)
