"""Build recipes for the checker side of the repository (test infrastructure).

* ``build_oracle()`` compiles the C restatement of the reference algorithm
  (``oracle/fdtd_oracle.c``) twice, once with ``double`` and once with ``float``
  state, into ``oracle/_build/<machine>/liboracle64.so`` and ``liboracle32.so``.
  It needs only a C compiler and runs on any host (x86 container or the Arm
  GPU host).
* ``stage_reference()`` copies the reference's own solver sources, unchanged,
  from the reference tree into ``oracle/_ref/src/`` (git-ignored, so they are
  never part of the repository's history, but they travel with a copy of the
  working tree to a machine that has no reference tree).
* ``build_reference()`` compiles the reference's own CPU solver
  (``FDTD_CPU.cxx`` + ``FDTD_common.cxx``, unchanged) together with
  ``oracle/ref_driver.cpp`` into ``oracle/_ref/<machine>/ref_driver``.  The
  reference has an uninitialised loop index at ``FDTD_CPU.cxx:816``
  (``for(int freq_index; ...)``) whose value decides whether the far-field
  post-process runs.  Instead of editing the source, the compiler is asked to
  zero-initialise automatic variables (``-ftrivial-auto-var-init=zero``), which
  is exactly the one-token fix ``int freq_index = 0``.
* ``build_reference_gpu()`` compiles the reference's own GPU solver
  (``FDTD_GPU.cu`` + ``FDTD_common.cxx``, unchanged) for sm_103a together with
  ``oracle/ref_gpu_driver.cpp`` into ``oracle/_ref/<machine>/ref_gpu_driver``.
  Every reference translation unit is compiled with ``-include
  oracle/ref_gpu_guard.h``, which routes the solver's cudaMalloc / cudaFree /
  cudaMemcpy calls through the driver: each device allocation gets 64 KiB of
  guard space on both sides.  The guard exists because the reference's
  ``Field_reset`` kernel (``FDTD_GPU.cu:436-503``) runs on a 418 x 418 thread
  grid and zeroes CPML psi entries outside its arrays: up to 27 KiB past the
  end of ``Psi_ezy`` / ``Psi_hxy`` and 80 bytes before ``Psi_ezx``
  (``FDTD_GPU.cu:441-473`` against the allocations at ``:885-888``; the
  extents are recomputed in ``tests/test_oracle.py``).  With the guard those
  stray zeros land in padding, so the run stays inside its allocations and
  computes what the source intends.

Sources are read from the reference tree named by the environment variable
``TOMO_REFERENCE_TREE`` (default: the checkout path below), or,
where that tree is absent, from the staged copy.  Nothing in the product
imports this module; ``__graft_entry__.build()`` calls it so that the checker
exists wherever the tests run.
"""
from __future__ import annotations

import os
import platform
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
MACHINE = platform.machine() or "unknown"
BUILD_DIR = os.path.join(HERE, "_build", MACHINE)
REF_ROOT = os.path.join(HERE, "_ref")
REF_OUT = os.path.join(REF_ROOT, MACHINE)
STAGE_DIR = os.path.join(REF_ROOT, "src")
REFERENCE_TREE = os.environ.get("TOMO_REFERENCE_TREE", "/root/reference")
REF_FILES = ("FDTD_CPU.cxx", "FDTD_CPU.h", "FDTD_GPU.cu", "FDTD_GPU.cuh", "FDTD_common.cxx", "FDTD_common.hxx")
GUARD_BYTES = 64 * 1024


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        sys.stderr.write(proc.stdout + proc.stderr)
        raise RuntimeError("command failed: " + " ".join(cmd))


def _stale(target: str, sources: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def oracle_lib_path(bits: int) -> str:
    return os.path.join(BUILD_DIR, f"liboracle{bits}.so")


def build_oracle(force: bool = False) -> None:
    os.makedirs(BUILD_DIR, exist_ok=True)
    src = os.path.join(HERE, "fdtd_oracle.c")
    hdr = os.path.join(HERE, "fdtd_oracle.h")
    cc = os.environ.get("CC", "gcc")
    for bits, real in ((64, "double"), (32, "float")):
        out = oracle_lib_path(bits)
        if not force and not _stale(out, [src, hdr, __file__]):
            continue
        # -ffp-contract=off: no fused multiply-add, so the geometry tests
        # (ellipse rasterisation) round exactly like the device code, which
        # uses explicit _rn intrinsics.
        _run([cc, "-O2", "-std=c11", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math",
              f"-DORACLE_REAL={real}", f"-DORACLE_BITS={bits}", "-pthread",
              "-o", out, src, "-lm"])


def _tree_has_sources(path: str) -> bool:
    return all(os.path.isfile(os.path.join(path, f)) for f in REF_FILES)


def stage_reference() -> bool:
    """Copy the reference solver sources (unchanged) into the git-ignored
    staging directory; returns False when the reference tree is absent."""
    if not _tree_has_sources(REFERENCE_TREE):
        return False
    os.makedirs(STAGE_DIR, exist_ok=True)
    for f in REF_FILES:
        src, dst = os.path.join(REFERENCE_TREE, f), os.path.join(STAGE_DIR, f)
        if _stale(dst, [src]):
            shutil.copyfile(src, dst)
    return True


def reference_source_dir() -> str | None:
    """The reference tree if present, else the staged copy, else None."""
    if _tree_has_sources(REFERENCE_TREE):
        return REFERENCE_TREE
    if _tree_has_sources(STAGE_DIR):
        return STAGE_DIR
    return None


def reference_available() -> bool:
    return reference_source_dir() is not None


def ref_driver_path() -> str:
    return os.path.join(REF_OUT, "ref_driver")


def ref_driver_ftz_path() -> str:
    return os.path.join(REF_OUT, "ref_driver_ftz")


def ref_gpu_driver_path() -> str:
    return os.path.join(REF_OUT, "ref_gpu_driver")


def build_reference(force: bool = False, ftz: bool = False) -> bool:
    """Compile the reference CPU solver; returns False when no sources are
    available.  ``ftz`` builds the timing variant with ``-ffast-math``, whose
    start-up code flushes denormals to zero (the reference's fields decay
    through the denormal range, which costs several times the run time)."""
    tree = reference_source_dir()
    if tree is None:
        return False
    os.makedirs(REF_OUT, exist_ok=True)
    out = ref_driver_ftz_path() if ftz else ref_driver_path()
    srcs = [os.path.join(tree, "FDTD_CPU.cxx"), os.path.join(tree, "FDTD_common.cxx"),
            os.path.join(HERE, "ref_driver.cpp")]
    if not force and not _stale(out, srcs + [__file__]):
        return True
    cxx = os.environ.get("CXX", "g++")
    # The reference's own optimisation flags (CMakeLists.txt:9) minus -g/-Wall;
    # -msse3 only exists on x86.
    flags = ["-O3", "-funroll-loops", "-w", "-ftrivial-auto-var-init=zero", "-I" + tree]
    if MACHINE in ("x86_64", "AMD64"):
        flags.append("-msse3")
    if ftz:
        flags.append("-ffast-math")
    _run([cxx] + flags + ["-o", out] + srcs + ["-pthread"])
    return True


def _nvcc() -> str | None:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    return None


def build_reference_gpu(force: bool = False) -> bool:
    """Compile the reference GPU solver with the allocation guard; returns
    False when no sources (or no nvcc) are available."""
    tree = reference_source_dir()
    nvcc = _nvcc()
    if tree is None or nvcc is None:
        return False
    os.makedirs(REF_OUT, exist_ok=True)
    out = ref_gpu_driver_path()
    guard = os.path.join(HERE, "ref_gpu_guard.h")
    drv = os.path.join(HERE, "ref_gpu_driver.cpp")
    srcs = [os.path.join(tree, "FDTD_GPU.cu"), os.path.join(tree, "FDTD_common.cxx"), drv]
    if not force and not _stale(out, srcs + [guard, __file__]):
        return True
    _run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-w", "-std=c++17",
          "-I" + tree, "-include", guard, f"-DTOMO_REF_GUARD_BYTES={GUARD_BYTES}", "-o", out] + srcs)
    return True


def main() -> None:
    force = "--force" in sys.argv
    build_oracle(force=force)
    staged = stage_reference()
    ok = build_reference(force=force)
    print("oracle:", oracle_lib_path(64), oracle_lib_path(32))
    print("reference sources:", reference_source_dir(), "(staged)" if staged else "")
    print("reference CPU driver:", ref_driver_path() if ok else "unavailable (no reference sources)")
    if "--gpu" in sys.argv:
        okg = build_reference_gpu(force=force)
        print("reference GPU driver:", ref_gpu_driver_path() if okg else "unavailable")


if __name__ == "__main__":
    main()
