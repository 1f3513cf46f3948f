"""Build recipes for the checker side of the repository (test infrastructure).

* ``build_oracle()`` compiles the C restatement of the reference algorithm
  (``oracle/fdtd_oracle.c``) twice, once with ``double`` and once with ``float``
  state, into ``oracle/_build/liboracle64.so`` and ``liboracle32.so``.  It needs
  only a C compiler and runs on any host (x86 container or the Arm GPU host).
* ``build_reference()`` compiles the reference's own CPU solver
  (``FDTD_CPU.cxx`` + ``FDTD_common.cxx``, unchanged, read from the reference
  tree) together with ``oracle/ref_driver.cpp`` into ``oracle/_ref/ref_driver``.
  The reference has an uninitialised loop index at ``FDTD_CPU.cxx:816``
  (``for(int freq_index; ...)``) whose value decides whether the far-field
  post-process runs.  Instead of editing or copying the source, the compiler is
  asked to zero-initialise automatic variables
  (``-ftrivial-auto-var-init=zero``), which is exactly the one-token fix
  ``int freq_index = 0``.  Only the binary is written into ``oracle/_ref/``.

Nothing in the product imports this module; ``__graft_entry__.build()`` calls
it so that the checker exists wherever the tests run.
"""
from __future__ import annotations

import os
import platform
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
REF_OUT = os.path.join(HERE, "_ref")
REFERENCE_TREE = "/root/reference"


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


def reference_available() -> bool:
    return os.path.isfile(os.path.join(REFERENCE_TREE, "FDTD_CPU.cxx"))


def ref_driver_path() -> str:
    return os.path.join(REF_OUT, "ref_driver")


def build_reference(force: bool = False) -> bool:
    """Compile the reference CPU solver; returns False when the tree is absent."""
    if not reference_available():
        return False
    os.makedirs(REF_OUT, exist_ok=True)
    out = ref_driver_path()
    srcs = [os.path.join(REFERENCE_TREE, "FDTD_CPU.cxx"), os.path.join(REFERENCE_TREE, "FDTD_common.cxx"),
            os.path.join(HERE, "ref_driver.cpp")]
    if not force and not _stale(out, srcs + [__file__]):
        return True
    cxx = os.environ.get("CXX", "g++")
    # The reference's own optimisation flags (CMakeLists.txt:9) minus -g/-Wall;
    # -msse3 only exists on x86.
    flags = ["-O3", "-funroll-loops", "-w", "-ftrivial-auto-var-init=zero", "-I" + REFERENCE_TREE]
    if platform.machine() in ("x86_64", "AMD64"):
        flags.append("-msse3")
    _run([cxx] + flags + ["-o", out] + srcs)
    return True


def main() -> None:
    build_oracle(force="--force" in sys.argv)
    ok = build_reference(force="--force" in sys.argv)
    print("oracle:", oracle_lib_path(64), oracle_lib_path(32))
    print("reference:", ref_driver_path() if ok else "unavailable (reference tree absent)")


if __name__ == "__main__":
    main()
