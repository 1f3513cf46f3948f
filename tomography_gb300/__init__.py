"""tomography_gb300: GB300-native forward FDTD fitness path for microwave tomography.

Python mirror of the reference's operator interface.  The reference exposes
``double FDTD_GPU(const std::vector<double>&)`` (FDTD_GPU.cuh:8) and tao's
search drivers call it once per candidate (test.cxx:94-121).  Here the same
entry point is :func:`FDTD_GPU`, and the batched / serving interfaces of the
native library are exposed through :class:`Solver` (``forward``,
``fitness_batch``, ``submit`` / ``serve_step`` / ``poll`` / ``wait``).  The
search drivers that stand in for tao's are in :mod:`tomography_gb300.search`;
the legacy total-field far field is ``reference_spec().copy(total_field=1)``.
Everything runs in the native library ``_lib/libtomography_gb300.so``
(hand-written sm_103a CUDA kernels behind the C ABI of
``include/tomography.h``); there is no Python or CPU fallback: if the library
cannot be loaded, every call raises.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional, Sequence

import numpy as np

from .spec import Spec, MODE_REFERENCE_GPU, MODE_REFERENCE_CPU, MODE_BREAST, FP32, FP64, MAX_FREQS  # noqa: F401

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libtomography_gb300.so")

TOMO_OK = 0
TOMO_ENUMERIC = -4
STATUS_NAMES = {
    -1: "TOMO_EINVAL",
    -2: "TOMO_ENOMEM_BUDGET",
    -3: "TOMO_ETIMEOUT",
    -4: "TOMO_ENUMERIC",
    -5: "TOMO_ECUDA",
    -6: "TOMO_ENOTREADY",
    -7: "TOMO_ECANCELLED",
    -8: "TOMO_ENOTARGET",
    -9: "TOMO_ENOMEM_HOST",
}


class TomoError(RuntimeError):
    """A non-OK status from the native library."""

    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


class Outputs(C.Structure):
    _fields_ = [
        ("traces", C.POINTER(C.c_float)),
        ("D", C.POINTER(C.c_float)),
        ("P", C.POINTER(C.c_float)),
        ("fitness", C.POINTER(C.c_double)),
        ("traces_f64", C.POINTER(C.c_double)),
    ]


class Stats(C.Structure):
    _fields_ = [
        ("advance_ms", C.c_double),
        ("total_ms", C.c_double),
        ("cell_updates", C.c_double),
        ("launches", C.c_int64),
        ("kernels", C.c_int64),
        ("steps_per_launch", C.c_int32),
        ("cols_per_lane", C.c_int32),
        ("h2d_bytes", C.c_int64),
        ("d2h_bytes", C.c_int64),
        ("tune_ms", C.c_double),
        ("tuned_configs", C.c_int32),
        ("min_blocks_per_sm", C.c_int32),
        ("serve_bytes_in_use", C.c_uint64),
        ("serve_running", C.c_int32),
        ("serve_queued", C.c_int32),
        ("serve_running_solves", C.c_int32),
    ]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


_lib: Optional[C.CDLL] = None


class SearchParams(C.Structure):
    """Mirror of tomo_search_params (search drivers, tomography_gb300.search)."""
    _fields_ = [
        ("type", C.c_int32), ("population_size", C.c_int32), ("maximum_iterations", C.c_int32),
        ("number_pairs", C.c_int32), ("seed", C.c_uint64),
        ("inertia", C.c_double), ("local_best_weight", C.c_double), ("global_best_weight", C.c_double),
        ("crossover_rate", C.c_double), ("differential_scale", C.c_double),
        ("parent_best", C.c_int32), ("reserved", C.c_int32),
        ("radius", C.POINTER(C.c_double)), ("regression_size", C.c_int32), ("line_search_size", C.c_int32),
        ("line_search_min", C.c_double), ("line_search_max", C.c_double), ("hessian_diagonal", C.c_int32),
        ("reserved2", C.c_int32),
    ]


# tomo_batch_fitness_fn and tomo_generation_fn
BATCH_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.POINTER(C.c_double), C.c_size_t, C.c_size_t, C.POINTER(C.c_double))
REPORT_FN = C.CFUNCTYPE(None, C.c_void_p, C.c_int, C.c_double, C.POINTER(C.c_double))


def library() -> C.CDLL:
    """Load the native library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"native library missing: {LIB_PATH} (run __graft_entry__.build())")
    lib = C.CDLL(LIB_PATH)
    P, I, SZ = C.c_void_p, C.c_int, C.c_size_t
    dp, fp = C.POINTER(C.c_double), C.POINTER(C.c_float)
    sig = {
        "tomo_spec_reference": (I, [C.POINTER(Spec), I]),
        "tomo_spec_breast": (I, [C.POINTER(Spec), I]),
        "tomo_spec_serving": (I, [C.POINTER(Spec), I, I]),
        "tomo_num_params": (I, [C.POINTER(Spec)]),
        "tomo_num_excitations": (I, [C.POINTER(Spec)]),
        "tomo_create": (I, [C.POINTER(Spec), C.POINTER(P)]),
        "tomo_destroy": (None, [P]),
        "tomo_set_stream": (I, [P, P]),
        "tomo_set_memory_budget": (I, [P, C.c_uint64]),
        "tomo_set_target": (I, [P, fp, SZ]),
        "tomo_fitness": (I, [P, dp, SZ, dp]),
        "tomo_fitness_batch": (I, [P, dp, SZ, SZ, dp]),
        "tomo_forward": (I, [P, dp, SZ, SZ, C.POINTER(Outputs)]),
        "tomo_submit": (I, [P, dp, SZ, SZ, C.POINTER(C.c_uint64)]),
        "tomo_submit_spec": (I, [P, C.POINTER(Spec), dp, SZ, SZ, C.POINTER(C.c_uint64)]),
        "tomo_set_target_spec": (I, [P, C.POINTER(Spec), fp, SZ]),
        "tomo_serve_step": (I, [P, C.POINTER(C.c_int)]),
        "tomo_poll": (I, [P, C.c_uint64, dp]),
        "tomo_wait": (I, [P, C.c_uint64, C.c_double, dp]),
        "tomo_request_bytes": (I, [P, C.c_void_p, SZ, C.POINTER(C.c_uint64)]),
        "tomo_cancel": (I, [P, C.c_uint64]),
        "tomo_get_stats": (I, [P, C.POINTER(Stats)]),
        "tomo_field_snapshot": (I, [P, SZ, I, I, fp, SZ]),
        "tomo_trace_misfit_static": (I, [C.c_void_p, C.c_void_p, SZ, SZ, SZ, C.c_void_p, C.c_void_p]),
        "tomo_search_defaults": (I, [C.POINTER(SearchParams), I]),
        "tomo_search_parse_args": (I, [C.POINTER(SearchParams), I, C.POINTER(C.c_char_p)]),
        "tomo_search_run": (I, [C.POINTER(SearchParams), dp, dp, SZ, BATCH_FN, P, REPORT_FN, P, dp, dp, dp,
                                C.POINTER(C.c_int64)]),
        "tomo_search_fitness": (I, [P, C.POINTER(SearchParams), dp, dp, REPORT_FN, P, dp, dp, dp]),
        "tomo_last_error": (C.c_char_p, []),
        "tomo_version": (C.c_char_p, []),
        "tomo_fdtd_gpu_set_target": (I, [fp, SZ]),
        "tomo_fdtd_gpu_release": (None, []),
        "tomo_internal_read_target_file": (I, [C.c_char_p, fp, SZ]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def _check(rc: int) -> None:
    if rc != TOMO_OK:
        raise TomoError(rc, library().tomo_last_error().decode())


def _dptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _fptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def reference_spec(cpu_variant: bool = False) -> Spec:
    """The reference's compile-time problem (FDTD_common.hxx:1-76) as a runtime spec."""
    s = Spec()
    _check(library().tomo_spec_reference(C.byref(s), 1 if cpu_variant else 0))
    return s


def breast_spec(config: int) -> Spec:
    """Breast-imaging workload presets 0..4."""
    s = Spec()
    _check(library().tomo_spec_breast(C.byref(s), int(config)))
    return s


def save_field(path: str, field: np.ndarray) -> None:
    """Write a field snapshot: ``.npy`` keeps the values; ``.pgm`` writes an 8-bit
    grey image with zero at mid-grey, scaled to the largest magnitude."""
    a = np.asarray(field, dtype=np.float32)
    if path.endswith(".npy"):
        np.save(path, a)
        return
    if not path.endswith(".pgm"):
        raise ValueError("field snapshots are written as .npy or .pgm")
    peak = float(np.abs(a).max()) or 1.0
    img = np.clip(np.rint(127.5 + 127.5 * a / peak), 0, 255).astype(np.uint8)[::-1]   # y up
    with open(path, "wb") as fp:
        fp.write(b"P5\n%d %d\n255\n" % (img.shape[1], img.shape[0]))
        fp.write(img.tobytes())


def serving_spec(edge: int, n_antennas: int) -> Spec:
    """One request of the serving workload: edge x edge cells over a 100 mm
    domain (breast at 70%), 4*edge steps, every antenna transmitting."""
    s = Spec()
    _check(library().tomo_spec_serving(C.byref(s), int(edge), int(n_antennas)))
    return s


class Solver:
    """One device-resident solver instance (C handle) for one problem spec."""

    def __init__(self, spec: Spec, stream: Optional[int] = None):
        lib = library()
        self.spec = Spec()
        C.memmove(C.byref(self.spec), C.byref(spec), C.sizeof(Spec))
        h = C.c_void_p()
        _check(lib.tomo_create(C.byref(self.spec), C.byref(h)))
        self._h = h
        self.n_params = lib.tomo_num_params(C.byref(self.spec))
        self.n_exc = lib.tomo_num_excitations(C.byref(self.spec))
        if stream is not None:
            self.set_stream(stream)

    def close(self) -> None:
        if getattr(self, "_h", None):
            library().tomo_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- configuration
    def set_stream(self, stream: int) -> None:
        _check(library().tomo_set_stream(self._h, C.c_void_p(stream)))

    def set_memory_budget(self, nbytes: int) -> None:
        _check(library().tomo_set_memory_budget(self._h, C.c_uint64(int(nbytes))))

    def set_target(self, target: np.ndarray) -> None:
        t = np.ascontiguousarray(target, dtype=np.float32).ravel()
        _check(library().tomo_set_target(self._h, _fptr(t), t.size))

    # -- evaluation
    def _args(self, args) -> np.ndarray:
        a = np.ascontiguousarray(args, dtype=np.float64)
        if a.ndim == 1:
            a = a[None, :]
        if a.shape[1] != self.n_params:
            raise ValueError(f"expected {self.n_params} parameters per candidate, got {a.shape[1]}")
        return a

    def fitness(self, args: Sequence[float]) -> float:
        a = self._args(args)
        out = np.zeros(1, dtype=np.float64)
        _check(library().tomo_fitness(self._h, _dptr(a), a.shape[1], _dptr(out)))
        return float(out[0])

    def fitness_batch(self, args, out: Optional[np.ndarray] = None, *, diverged: str = "raise") -> np.ndarray:
        """Fitness of every candidate of ``args`` ([n_cand, n_params]).  A
        candidate whose solve diverges has a non-finite fitness: ``diverged=
        "raise"`` raises TomoError(TOMO_ENUMERIC); ``"keep"`` returns every
        fitness, the diverged ones non-finite (what a search wants: the
        reference's search goes on past a clamped field)."""
        if diverged not in ("raise", "keep"):
            raise ValueError("diverged must be 'raise' or 'keep'")
        a = self._args(args)
        if out is None:
            out = np.zeros(a.shape[0], dtype=np.float64)
        rc = library().tomo_fitness_batch(self._h, _dptr(a), a.shape[0], a.shape[1], _dptr(out))
        if not (rc == TOMO_ENUMERIC and diverged == "keep"):
            _check(rc)
        return out

    def forward(self, args, traces: bool = True, far_field: bool = True, fitness: bool = False,
                traces_f64: bool = False) -> dict:
        """Forward solves of a batch; returns numpy arrays of the requested outputs."""
        a = self._args(args)
        n = a.shape[0]
        s = self.spec
        res: dict = {}
        o = Outputs()
        if traces and s.mode == MODE_BREAST:
            res["traces"] = np.zeros((n, self.n_exc, s.n_antennas, s.steps), dtype=np.float32)
            o.traces = _fptr(res["traces"])
        if traces_f64 and s.mode == MODE_BREAST:
            res["traces_f64"] = np.zeros((n, self.n_exc, s.n_antennas, s.steps), dtype=np.float64)
            o.traces_f64 = _dptr(res["traces_f64"])
        if far_field and s.nfreq > 0:
            res["D"] = np.zeros((n, self.n_exc, s.nfreq, s.n_angles), dtype=np.float32)
            res["P"] = np.zeros_like(res["D"])
            o.D = _fptr(res["D"])
            o.P = _fptr(res["P"])
        if fitness:
            res["fitness"] = np.zeros(n, dtype=np.float64)
            o.fitness = _dptr(res["fitness"])
        _check(library().tomo_forward(self._h, _dptr(a), n, a.shape[1], C.byref(o)))
        return res

    # -- serving
    def submit(self, args, spec: Optional[Spec] = None) -> int:
        """Queue a request; ``spec`` may select another grid (same precision)."""
        a = np.ascontiguousarray(args, dtype=np.float64)
        if a.ndim == 1:
            a = a[None, :]
        t = C.c_uint64()
        if spec is None:
            a = self._args(a)
            _check(library().tomo_submit(self._h, _dptr(a), a.shape[0], a.shape[1], C.byref(t)))
        else:
            _check(library().tomo_submit_spec(self._h, C.byref(spec), _dptr(a), a.shape[0], a.shape[1], C.byref(t)))
        return int(t.value)

    def set_target_for(self, spec: Spec, target: np.ndarray) -> None:
        t = np.ascontiguousarray(target, dtype=np.float32).ravel()
        _check(library().tomo_set_target_spec(self._h, C.byref(spec), _fptr(t), t.size))

    def request_bytes(self, n_cand: int, spec: Optional[Spec] = None) -> int:
        """Device bytes a request of n_cand candidates holds while admitted (what
        the memory budget is charged)."""
        b = C.c_uint64()
        sp = C.cast(C.byref(spec), C.c_void_p) if spec is not None else None
        _check(library().tomo_request_bytes(self._h, sp, int(n_cand), C.byref(b)))
        return int(b.value)

    def serve_step(self) -> int:
        n = C.c_int()
        _check(library().tomo_serve_step(self._h, C.byref(n)))
        return int(n.value)

    def poll(self, ticket: int, n_cand: int) -> Optional[np.ndarray]:
        out = np.zeros(n_cand, dtype=np.float64)
        rc = library().tomo_poll(self._h, C.c_uint64(ticket), _dptr(out))
        if rc == -6:
            return None
        _check(rc)
        return out

    def wait(self, ticket: int, n_cand: int, timeout_s: float) -> np.ndarray:
        """Drive the serving loop until `ticket` finishes (its fitness) or
        `timeout_s` passes (TomoError with status TOMO_ETIMEOUT; the request
        stays queued or running)."""
        out = np.zeros(n_cand, dtype=np.float64)
        _check(library().tomo_wait(self._h, C.c_uint64(ticket), C.c_double(timeout_s * 1e3), _dptr(out)))
        return out

    def cancel(self, ticket: int) -> None:
        _check(library().tomo_cancel(self._h, C.c_uint64(ticket)))

    FIELDS = {"ez": 0, "hx": 1, "hy": 2}

    def field_snapshot(self, candidate: int = 0, excitation: int = 0, field: str = "ez") -> np.ndarray:
        """Final Ez ((ny+1) x (nx+1)), Hx or Hy (ny x nx) of one solve of the last
        batch, as float32 [y][x]."""
        f = self.FIELDS[field.lower()]
        nx, ny = self.spec.nx, self.spec.ny
        out = np.zeros((ny + 1, nx + 1) if f == 0 else (ny, nx), dtype=np.float32)
        _check(library().tomo_field_snapshot(self._h, int(candidate), int(excitation), f, _fptr(out), out.size))
        return out

    def stats(self) -> dict:
        st = Stats()
        _check(library().tomo_get_stats(self._h, C.byref(st)))
        return st.as_dict()


_dropin: Optional[Solver] = None
REFERENCE_TARGET_SIZE = 4000   # E * F * A of the reference preset (4 x 10 x 100)


def target_shape(spec: Spec) -> tuple:
    """Shape of the target Solver.set_target takes for spec: the receiver
    traces [n_tx][n_antennas][steps] in the breast mode, the far-field
    magnitudes [n_excitations][nfreq][n_angles] in the reference modes."""
    if spec.mode == MODE_BREAST:
        return (spec.n_tx, spec.n_antennas, spec.steps)
    return (library().tomo_num_excitations(C.byref(spec)), spec.nfreq, spec.n_angles)


def save_target(path: str, target: np.ndarray) -> None:
    """Write a target: NumPy .npy when path ends in .npy, text (one value per
    line) for .txt and .csv, else raw little-endian float32."""
    t = np.ascontiguousarray(target, dtype=np.float32)
    low = path.lower()
    if low.endswith(".npy"):
        np.save(path, t)
    elif low.endswith((".txt", ".csv")):
        np.savetxt(path, t.ravel(), fmt="%.9g")
    else:
        t.ravel().astype("<f4").tofile(path)


def load_target(path: str, spec: Spec) -> np.ndarray:
    """Read a target for spec from a file in one of save_target's formats:
    .npy (any real dtype), text (.txt/.csv: numbers separated by spaces,
    commas or newlines; anything else raises) or raw little-endian float32.
    It must hold exactly the target's number of values, or in the reference
    modes twice that (magnitudes then phases, the reference's whole array),
    of which the first half is used.  Returns float32 in target_shape(spec)."""
    import re

    shape = target_shape(spec)
    n = int(np.prod(shape))
    low = path.lower()
    if low.endswith(".npy"):
        v = np.load(path, allow_pickle=False)
        if not np.issubdtype(v.dtype, np.floating) and not np.issubdtype(v.dtype, np.integer):
            raise ValueError(f"{path}: not a real-valued array")
        v = v.astype(np.float64).ravel()
    elif low.endswith((".txt", ".csv")):
        with open(path, encoding="utf-8-sig") as fp:
            tokens = [t for t in re.split(r"[\s,]+", fp.read().strip()) if t]
        try:
            v = np.array([float(t) for t in tokens])
        except ValueError as e:
            raise ValueError(f"{path}: {e}") from None
    else:
        raw = np.fromfile(path, dtype=np.uint8)
        if raw.size % 4:
            raise ValueError(f"{path}: {raw.size} bytes is not a whole number of float32 values")
        v = raw.view("<f4").astype(np.float64)
    if v.size == 2 * n and spec.mode != MODE_BREAST:
        v = v[:n]
    if v.size != n:
        raise ValueError(f"{path}: {v.size} values, the target of this spec holds {n} {shape}")
    if not np.all(np.isfinite(v)):
        raise ValueError(f"{path}: non-finite values")
    return v.astype(np.float32).reshape(shape)


def read_target_file(path: str) -> np.ndarray:
    """The far-field target of the drop-in from a measurement file, with the
    native library's rules: raw float32 or text (numbers separated by spaces,
    commas or newlines), 4000 values or 8000 (magnitudes then phases) of which
    the first 4000 are used; a .npy file or any other content raises."""
    out = np.zeros(REFERENCE_TARGET_SIZE, dtype=np.float32)
    n = library().tomo_internal_read_target_file(path.encode(), _fptr(out), out.size)
    _check(n if n < 0 else TOMO_OK)
    return out[:n]


def _target_values(measurement) -> np.ndarray:
    m = np.ascontiguousarray(measurement, dtype=np.float32).ravel()
    if m.size not in (REFERENCE_TARGET_SIZE, 2 * REFERENCE_TARGET_SIZE):
        raise TomoError(-1, f"the target needs {REFERENCE_TARGET_SIZE} values (or {2 * REFERENCE_TARGET_SIZE}: "
                            f"magnitudes then phases), got {m.size}")
    return m[:REFERENCE_TARGET_SIZE]


def FDTD_GPU(arguments: Sequence[float], measurement: Optional[np.ndarray] = None) -> float:
    """Drop-in for ``double FDTD_GPU(const std::vector<double>&)`` (FDTD_GPU.cuh:8).

    ``arguments``: 27 values, eps_inf of the 3x3 patches, then del_eps, then
    sigma (FDTD_GPU.cu:657-693).  Raises IndexError for a short vector (the
    reference's ``.at()`` throws std::out_of_range).  The far-field target is
    ``measurement`` (4000 magnitudes, or the reference's whole 8000-entry
    array) or the file named by TOMO_MEASUREMENT_FILE (see read_target_file).
    """
    global _dropin
    args = [float(v) for v in arguments]
    if len(args) < 27:
        raise IndexError("FDTD_GPU: expected 27 arguments")
    if _dropin is None:
        solver = Solver(reference_spec(False))
        if measurement is None:
            path = os.environ.get("TOMO_MEASUREMENT_FILE")
            if not path:
                raise TomoError(-8, "no target: pass measurement= or set TOMO_MEASUREMENT_FILE")
            measurement = read_target_file(path)
        solver.set_target(_target_values(measurement))
        _dropin = solver
    elif measurement is not None:
        _dropin.set_target(_target_values(measurement))
    return _dropin.fitness(args[:27])
