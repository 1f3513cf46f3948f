"""Python side of the CPU oracle (checker only; see fdtd_oracle.h).

Builds oracle problems from a spec dictionary (``Spec.as_dict()`` of the
product, i.e. plain numbers) and runs the C restatement.  Everything derived
from the spec -- CPML profile, material coefficients, patch / ellipse maps,
antenna cells, source waveform, contour, far field, misfits -- is recomputed
here or in fdtd_oracle.c from the reference formulas, independently of the
product code.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
if HERE not in sys.path:
    sys.path.insert(0, HERE)
import build as _build  # noqa: E402

PI = 3.141592653589793238
MU0 = PI * 4e-7
EPS0 = 8.85418e-12
C0 = 1.0 / math.sqrt(MU0 * EPS0)
ETA0 = math.sqrt(MU0 / EPS0)
NCOEF = 8
REF_CPML, NAN_CLAMP, PLANE_WAVE, M_LAG, TOTAL_FIELD = 1, 2, 4, 8, 16

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_ubp = C.POINTER(C.c_ubyte)


class OracleProblem(C.Structure):
    _fields_ = [
        ("nx", C.c_int), ("ny", C.c_int), ("steps", C.c_int), ("ncpml", C.c_int),
        ("flags", C.c_int), ("nmat", C.c_int),
        ("dx", C.c_double), ("dt", C.c_double), ("chez", C.c_double), ("Kp", C.c_double),
        ("cpml", _dp), ("mat", _ubp), ("mtab", _dp),
        ("pw_kx", C.c_double), ("pw_ky", C.c_double), ("pw_xoff", C.c_double), ("pw_yoff", C.c_double),
        ("pw_t0", C.c_double), ("pw_tau", C.c_double), ("pw_l", C.c_double), ("pw_c0", C.c_double),
        ("src_x", C.c_int), ("src_y", C.c_int), ("src_wave", _dp),
        ("nrx", C.c_int), ("rx", _ip), ("traces", _dp),
        ("nf_d", C.c_int), ("nfreq", C.c_int), ("freqs", _dp), ("acc", _dp),
        ("ez_out", _dp), ("hx_out", _dp), ("hy_out", _dp), ("jp_out", _dp),
        ("inc_x", C.c_int), ("inc_y", C.c_int), ("inc_wave", _dp), ("inc_acc", _dp),
    ]


_libs: dict = {}


def lib(bits: int = 64) -> C.CDLL:
    if bits not in _libs:
        _build.build_oracle()
        L = C.CDLL(_build.oracle_lib_path(bits))
        L.oracle_solve.argtypes = [C.POINTER(OracleProblem)]
        L.oracle_solve_many.argtypes = [C.POINTER(OracleProblem), C.c_int, C.c_int]
        L.oracle_contour_size.argtypes = [C.c_int, C.c_int, C.c_int]
        L.oracle_contour_point.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, _ip, _ip, _ip]
        L.oracle_far_field.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_int, _dp, _dp, C.c_int, C.c_int,
                                       C.c_double, C.c_double, _dp, _dp]
        L.oracle_cpml_profile.argtypes = [C.c_int, C.c_double, C.c_double, C.c_double, C.c_double, C.c_double,
                                          C.c_double, C.c_double, _dp]
        L.oracle_material_coefs.argtypes = [C.c_double] * 6 + [_dp, _dp]
        L.oracle_patch_map.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_int, _ubp]
        L.oracle_ellipse_map.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_int, _dp, _ubp]
        _libs[bits] = L
    return _libs[bits]


def _d(a):
    return a.ctypes.data_as(_dp)


# ----------------------------------------------------------------- precompute
def cpml_profile(spec: dict) -> np.ndarray:
    nc = spec["ncpml"]
    out = np.zeros(6 * max(nc, 1))
    lib().oracle_cpml_profile(nc, spec["cpml_grading"], spec["cpml_sigma_max"], spec["cpml_kappa_max"],
                              spec["cpml_alpha_max"], spec["cpml_alpha_min"], spec["dx"], spec["dt"], _d(out))
    return out


def material_coefs(eps_inf: float, del_eps: float, sigma: float, spec: dict) -> tuple[np.ndarray, float]:
    out = np.zeros(NCOEF)
    kp = C.c_double()
    lib().oracle_material_coefs(eps_inf, del_eps, sigma, spec["tau"], spec["dt"], spec["dx"], _d(out), C.byref(kp))
    return out, kp.value


def contour_size(nx: int, ny: int, d: int) -> int:
    return lib().oracle_contour_size(nx, ny, d)


def antenna_cells(spec: dict) -> np.ndarray:
    n = spec["n_antennas"]
    cells = []
    for a in range(n):
        th = 2 * PI * a / n
        x = spec["nx"] / 2.0 + (spec["antenna_radius"] / spec["dx"]) * math.cos(th)
        y = spec["ny"] / 2.0 + (spec["antenna_radius"] / spec["dx"]) * math.sin(th)
        # C lround: half away from zero
        cells.append((int(math.floor(x + 0.5)) if x >= 0 else -int(math.floor(-x + 0.5)),
                      int(math.floor(y + 0.5)) if y >= 0 else -int(math.floor(-y + 0.5))))
    return np.array(cells, dtype=np.int32)


def source_wave(spec: dict) -> np.ndarray:
    amp = spec["src_amp"] or (2 * spec["bg_eps_inf"] * EPS0 + spec["bg_sigma"] * spec["dt"]) / (2 * spec["dt"])
    t = (np.arange(spec["steps"]) + 0.5) * spec["dt"] - spec["src_t0"]
    return amp * np.sin(2 * PI * spec["src_f0"] * t) * np.exp(-(t / spec["src_tau"]) ** 2)


def incident_wave(spec: dict, steps: int | None = None) -> np.ndarray:
    """Point source of the legacy incident grid, added to its Ez in step n:
    100 Cezj fwf(n, 0, 0, 0, 0) with Cezj = -dt/eps0 (oldFDTD_GPU.cu:666,682) and
    fwf at the origin with angle 0 and offset 0: exp(-((n dt - t0)/tau)^2)
    (oldFDTD_GPU.cu:351-364), t0 and tau of the plane wave."""
    S = spec["steps"] if steps is None else steps
    t = np.arange(S) * spec["dt"] - spec["pw_t0"]
    return 100.0 * (-spec["dt"] / EPS0) * np.exp(-(t / spec["pw_tau"]) ** 2)


def material_table_reference(args: np.ndarray, spec: dict) -> tuple[np.ndarray, float]:
    """(nmat x NCOEF) table: material 0 vacuum, 1+p patch p (FDTD_GPU.cu:657-743 /
    FDTD_CPU.cxx:682-698, arguments rounded to float as the reference does)."""
    np2 = spec["npatch"] ** 2
    a = np.asarray(args, dtype=np.float64).astype(np.float32).astype(np.float64)
    rows, kp = [], None
    c, kp = material_coefs(1.0, 0.0, 0.0, spec)
    rows.append(c)
    for p in range(np2):
        if spec["mode"] == 0:
            c, kp = material_coefs(a[p], a[np2 + p], a[2 * np2 + p], spec)
        else:
            c, kp = material_coefs(a[p], 0.0, a[np2 + p], spec)
        rows.append(c)
    return np.array(rows), kp


def patch_map(spec: dict) -> np.ndarray:
    nx, ny = spec["nx"], spec["ny"]
    m = np.zeros((ny + 1) * (nx + 1), dtype=np.uint8)
    lib().oracle_patch_map(nx, ny, spec["dx"], spec["breast_radius"], spec["npatch"], m.ctypes.data_as(_ubp))
    return m


def ellipse_geometry(params: np.ndarray) -> np.ndarray:
    """(K, 6) = (cx, cy, a, b, cos, sin); math.cos/sin call the C library."""
    p = np.asarray(params, dtype=np.float64).reshape(-1, 8)
    return np.array([[e[0], e[1], e[2], e[3], math.cos(e[4]), math.sin(e[4])] for e in p]).reshape(-1, 6)


def ellipse_map(spec: dict, params: np.ndarray) -> np.ndarray:
    nx, ny = spec["nx"], spec["ny"]
    geo = np.ascontiguousarray(ellipse_geometry(params))
    m = np.zeros((ny + 1) * (nx + 1), dtype=np.uint8)
    lib().oracle_ellipse_map(nx, ny, spec["dx"], spec["disc_radius"], geo.shape[0], _d(geo), m.ctypes.data_as(_ubp))
    return m


def material_table_breast(params: np.ndarray, spec: dict) -> tuple[np.ndarray, float]:
    p = np.asarray(params, dtype=np.float64).reshape(-1, 8)
    rows = []
    c, kp = material_coefs(spec["bg_eps_inf"], spec["bg_del_eps"], spec["bg_sigma"], spec)
    rows.append(c)
    c, kp = material_coefs(spec["disc_eps_inf"], spec["disc_del_eps"], spec["disc_sigma"], spec)
    rows.append(c)
    for e in p:
        c, kp = material_coefs(e[5], e[6], e[7], spec)
        rows.append(c)
    return np.array(rows), kp


# ----------------------------------------------------------------- problems
class Problem:
    """An oracle_problem plus the numpy arrays it points into."""

    def __init__(self, spec: dict, steps: int | None = None):
        self.spec = spec
        self.keep = []
        self.p = OracleProblem()
        p = self.p
        p.nx, p.ny = spec["nx"], spec["ny"]
        p.steps = spec["steps"] if steps is None else steps
        p.ncpml = spec["ncpml"]
        p.dx, p.dt = spec["dx"], spec["dt"]
        p.chez = (spec["dt"] / spec["dx"]) / MU0
        p.src_x = p.src_y = -1
        self._arr("cpml", cpml_profile(spec))

    def _arr(self, field: str, a: np.ndarray, ctype=_dp):
        a = np.ascontiguousarray(a)
        self.keep.append(a)
        setattr(self.p, field, a.ctypes.data_as(ctype))
        return a

    def set_materials(self, mat: np.ndarray, tab: np.ndarray, kp: float):
        self.mat = self._arr("mat", mat.astype(np.uint8), _ubp)
        self.p.nmat = tab.shape[0]
        self._arr("mtab", tab.astype(np.float64))
        self.p.Kp = kp

    def want_traces(self, rx: np.ndarray):
        self.p.nrx = rx.shape[0]
        self._arr("rx", rx.astype(np.int32).ravel(), _ip)
        self.traces = self._arr("traces", np.zeros((rx.shape[0], self.p.steps)))

    def want_dft(self, d: int, freqs):
        self.p.nf_d = d
        self.p.nfreq = len(freqs)
        self._arr("freqs", np.array(freqs, dtype=np.float64))
        C_ = contour_size(self.p.nx, self.p.ny, d)
        self.acc = self._arr("acc", np.zeros((len(freqs), C_, 4)))

    def want_fields(self):
        nx, ny = self.p.nx, self.p.ny
        self.ez = self._arr("ez_out", np.zeros((ny + 1, nx + 1)))
        self.jp = self._arr("jp_out", np.zeros((ny + 1, nx + 1)))
        self.hx = self._arr("hx_out", np.zeros((ny, nx)))
        self.hy = self._arr("hy_out", np.zeros((ny, nx)))


def reference_problem(spec: dict, args: np.ndarray, exc: int, steps: int | None = None) -> Problem:
    """One plane-wave excitation of the reference modes (FDTD_GPU.cu:937-985 /
    FDTD_CPU.cxx:799-840)."""
    pr = Problem(spec, steps)
    tab, kp = material_table_reference(args, spec)
    pr.set_materials(patch_map(spec), tab, kp)
    p = pr.p
    p.flags = REF_CPML | PLANE_WAVE | (NAN_CLAMP if spec["nan_clamp"] else 0)
    phi = float(np.float32(exc * 2 * PI / spec["n_excitations"]))
    p.pw_kx, p.pw_ky = math.cos(phi), math.sin(phi)
    off = spec["nx"] // 2 if spec["pw_centred"] else 0
    p.pw_xoff = p.pw_yoff = float(off)
    p.pw_t0, p.pw_tau, p.pw_l, p.pw_c0 = spec["pw_t0"], spec["pw_tau"], spec["pw_l"], C0
    if spec["nfreq"] > 0:
        pr.want_dft(spec["nf2ff_d"], spec["freqs"])
    if spec.get("total_field"):
        # legacy total-field NTFF: incident grid with the source at the centre
        # (oldFDTD_GPU.cu:74-75 source_x = nx/2, source_y = ny/2)
        p.flags |= TOTAL_FIELD
        p.inc_x, p.inc_y = spec["nx"] // 2, spec["ny"] // 2
        pr._arr("inc_wave", incident_wave(spec, p.steps))
        if spec["nfreq"] > 0:
            pr.inc_acc = pr._arr("inc_acc", np.zeros_like(pr.acc))
    return pr


def breast_problem(spec: dict, params: np.ndarray, tx: int, steps: int | None = None) -> Problem:
    """One transmitter of the breast-imaging mode."""
    pr = Problem(spec, steps)
    tab, kp = material_table_breast(params, spec)
    pr.set_materials(ellipse_map(spec, params), tab, kp)
    ant = antenna_cells(spec)
    p = pr.p
    p.flags = 0
    p.src_x, p.src_y = int(ant[tx, 0]), int(ant[tx, 1])
    pr._arr("src_wave", source_wave(spec)[: p.steps].copy())
    pr.want_traces(ant)
    if spec["nfreq"] > 0:
        pr.want_dft(spec["nf2ff_d"], spec["freqs"])
    return pr


def run(problems: list, bits: int = 64, threads: int | None = None) -> None:
    arr = (OracleProblem * len(problems))(*[pr.p for pr in problems])
    n = threads or min(len(problems), os.cpu_count() or 1)
    rc = lib(bits).oracle_solve_many(arr, len(problems), n)
    if rc != 0:
        raise RuntimeError("oracle_solve_many failed")


def far_field(pr: Problem, norm: int, tau: float, nangle: int, bits: int = 64) -> tuple[np.ndarray, np.ndarray]:
    s = pr.spec
    F = pr.p.nfreq
    D = np.zeros((F, nangle))
    P = np.zeros((F, nangle))
    freqs = np.array(s["freqs"][:F], dtype=np.float64)
    # the breast mode's contour lies in its lossless background (refractive
    # index sqrt(bg_eps_inf)); the reference modes transform in vacuum
    nbg = math.sqrt(s["bg_eps_inf"]) if s.get("mode") == 2 else 1.0
    lib(bits).oracle_far_field(pr.p.nx, pr.p.ny, pr.p.nf_d, pr.p.dx, F, _d(freqs), _d(pr.acc), nangle, norm, tau,
                               nbg, _d(D), _d(P))
    return D, P


# ----------------------------------------------------------------- misfits
def misfit_abs(D: np.ndarray, m: np.ndarray, n_exc: int, nfreq: int) -> float:
    """FDTD_GPU.cu:1004-1022: -sum (D - m)^2 / (E F)."""
    D = np.asarray(D, dtype=np.float64).ravel()
    m = np.asarray(m, dtype=np.float64).ravel()[: D.size]
    return float(-np.sum((D - m) ** 2 / (n_exc * nfreq)))


def misfit_rel(D: np.ndarray, m: np.ndarray, n_exc: int, nfreq: int) -> float:
    """FDTD_CPU.cxx:841-845: -sum (D - m)^2 / (m^2 E F)."""
    D = np.asarray(D, dtype=np.float64).ravel()
    m = np.asarray(m, dtype=np.float64).ravel()[: D.size]
    return float(-np.sum((D - m) ** 2 / (m * m * n_exc * nfreq)))


def misfit_trace(traces: np.ndarray, target: np.ndarray) -> float:
    """-sum (s - t)^2 / sum t^2 over transmitters, receivers and steps."""
    s = np.asarray(traces, dtype=np.float64).ravel()
    t = np.asarray(target, dtype=np.float64).ravel()
    return float(-np.sum((s - t) ** 2) / np.sum(t * t))


# ----------------------------------------------------------------- whole evaluations
def reference_forward(spec: dict, args: np.ndarray, steps: int | None = None, bits: int = 64,
                      fields: bool = False) -> dict:
    """All excitations of one reference-mode candidate: D, P [E][F][A] and DFT accumulators."""
    E = spec["n_excitations"]
    probs = [reference_problem(spec, args, e, steps) for e in range(E)]
    if fields:
        for pr in probs:
            pr.want_fields()
    run(probs, bits)
    D = np.zeros((E, spec["nfreq"], spec["n_angles"]))
    P = np.zeros_like(D)
    for e, pr in enumerate(probs):
        D[e], P[e] = far_field(pr, spec["ff_norm"], spec["pw_tau"], spec["n_angles"], bits)
    return {"D": D, "P": P, "problems": probs}


def breast_forward(spec: dict, params: np.ndarray, steps: int | None = None, bits: int = 64,
                   txs=None, fields: bool = False) -> dict:
    txs = list(range(spec["n_tx"])) if txs is None else list(txs)
    probs = [breast_problem(spec, params, t, steps) for t in txs]
    if fields:
        for pr in probs:
            pr.want_fields()
    run(probs, bits)
    out = {"traces": np.stack([pr.traces for pr in probs]), "problems": probs}
    if spec["nfreq"] > 0:
        DP = [far_field(pr, spec["ff_norm"], spec["pw_tau"], spec["n_angles"], bits) for pr in probs]
        out["D"] = np.stack([d for d, _ in DP])
        out["P"] = np.stack([p for _, p in DP])
    return out


# ----------------------------------------------------------------- workload presets (checker side)
# The breast-imaging workloads restated here as plain numbers, so that the
# CPU baseline and the reference arm of the benchmark build their problems
# without loading the product library; tests/test_oracle.py checks them field
# by field against the product's presets.
def _breast_derived(s: dict) -> dict:
    s["dt"] = 0.99 * s["dx"] / (C0 * math.sqrt(2.0))
    s.update(cpml_grading=3.0, cpml_sigma_max=0.8 * 4 / (ETA0 * s["dx"]), cpml_kappa_max=5.0, cpml_alpha_max=0.05,
             cpml_alpha_min=0.0, tau=13e-12, bg_eps_inf=9.0, bg_del_eps=0.0, bg_sigma=0.0, src_f0=6e9)
    fmax = C0 / (20 * s["dx"] * math.sqrt(s["bg_eps_inf"]))
    band = max(fmax - s["src_f0"], 1e9)
    s["src_tau"] = math.sqrt(math.log(10.0)) / (PI * band)
    s.update(src_t0=4 * s["src_tau"], src_amp=0.0, nf2ff_d=s["ncpml"] + 3, ff_norm=0, misfit=2)
    return s


def breast_spec(config: int) -> dict:
    """Breast-imaging workload `config` (0: plain forward solve, 1: PSO
    generation, 2: precision study, 3: serving request, 4: large batch)."""
    s = dict(mode=2, precision=0, dx=0.5e-3, nx=200, ny=200, steps=1000, ncpml=10, n_ellipses=3, n_antennas=16,
             n_tx=1, antenna_radius=45e-3, nfreq=3, freqs=[3e9, 6e9, 9e9], n_angles=72, disc_radius=35e-3,
             disc_eps_inf=3.1, disc_del_eps=1.6, disc_sigma=0.036)
    if config == 1:
        s.update(nx=400, ny=400, ncpml=12, steps=3000, n_ellipses=8, n_tx=16)
    elif config == 2:
        s.update(nx=600, ny=600, dx=0.25e-3, ncpml=12, steps=6000, n_antennas=32, n_tx=32, antenna_radius=70e-3,
                 nfreq=8, freqs=[2e9 + 1e9 * f for f in range(8)], n_angles=360)
    elif config == 3:
        s.update(nx=256, ny=256, dx=0.1 / 256, ncpml=10, steps=4 * 256, n_ellipses=8, n_tx=16,
                 antenna_radius=42e-3)
    elif config == 4:
        s.update(nx=2048, ny=2048, dx=0.125e-3, ncpml=16, steps=20000, n_antennas=32, n_tx=32, n_ellipses=16,
                 antenna_radius=70e-3, disc_eps_inf=15.9, disc_del_eps=23.8, disc_sigma=0.83, nfreq=16,
                 freqs=[1e9 + 0.5e9 * f for f in range(16)], n_angles=720)
    elif config != 0:
        raise ValueError("breast config must be 0..4")
    return _breast_derived(s)


_MASK64 = (1 << 64) - 1


def _splitmix_uniforms(seed: int):
    """splitmix64 -> uniform doubles in [0, 1) (the workloads' seeded generator)."""
    state = seed & _MASK64
    while True:
        state = (state + 0x9E3779B97F4A7C15) & _MASK64
        z = state
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & _MASK64
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & _MASK64
        yield ((z ^ (z >> 31)) >> 11) * (1.0 / (1 << 53))


def candidate_params(seed: int, n_ellipses: int, disc_radius: float = 35e-3) -> np.ndarray:
    """One PSO candidate: per ellipse a centre uniform in the disc, semi-axes in
    [2, 15] mm, angle in [0, pi), eps_inf in [2, 20], del_eps in [1, 40],
    sigma in [0, 1] S/m."""
    u = _splitmix_uniforms(seed)
    out = []
    for _ in range(n_ellipses):
        r = disc_radius * math.sqrt(next(u))
        phi = 2 * math.pi * next(u)
        out += [r * math.cos(phi), r * math.sin(phi), 2e-3 + 13e-3 * next(u), 2e-3 + 13e-3 * next(u),
                math.pi * next(u), 2 + 18 * next(u), 1 + 39 * next(u), next(u)]
    return np.array(out, dtype=np.float64)


def workload_candidates(config: int, n_cand: int, n_ellipses: int, disc_radius: float = 35e-3) -> np.ndarray:
    """Candidates 0..n_cand-1 of workload `config` (seed 0x70F00000 + config + 1000 k)."""
    seed = 0x70F00000 + config
    return np.stack([candidate_params(seed + 1000 * k, n_ellipses, disc_radius) for k in range(n_cand)])
