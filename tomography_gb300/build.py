"""In-tree build of the native library ``tomography_gb300/_lib/libtomography_gb300.so``.

Each translation unit is compiled by nvcc for sm_103a only (GB300), in
parallel, then linked into one shared library that exports the C ABI of
``include/tomography.h`` and the C++ drop-in of ``include/tomography_fdtd.hpp``.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import platform
import shutil
import struct
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
# objects are kept per machine: a copy of the tree moved between an x86 build
# host and an Arm GPU host must never reuse the other's objects
OBJ_DIR = os.path.join(HERE, "_build", platform.machine() or "unknown")
LIB = os.path.join(OUT_DIR, "libtomography_gb300.so")
REPO = os.path.dirname(HERE)

SOURCES = [
    "advance_f32_b1.cu",
    "advance_f32_b2.cu",
    "advance_f32_b3.cu",
    "advance_f32_b4.cu",
    "advance_f32_ref.cu",
    "advance_f64.cu",
    "advance_registry.cu",
    "engine.cu",
    "serve.cu",
    "capi.cpp",
    "search.cpp",
    "fdtd_gpu_dropin.cpp",
    "noalloc.cu",
    "plain.cu",
]

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "--expt-relaxed-constexpr", "-I", os.path.join(REPO, "include")]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _deps() -> list[str]:
    """Every header a translation unit may include (csrc/*.h, *.cuh and the
    public include/ headers) and this script: a change to any of them
    rebuilds every object."""
    out = []
    for d, exts in ((CSRC, (".h", ".cuh", ".hpp")), (os.path.join(REPO, "include"), (".h", ".hpp"))):
        out += sorted(os.path.join(d, f) for f in os.listdir(d) if f.endswith(exts))
    out.append(__file__)
    return out


def _compile(src: str, extra: list[str]) -> str:
    obj = os.path.join(OBJ_DIR, os.path.basename(src) + ".o")
    srcp = os.path.join(CSRC, src)
    newest = max([os.path.getmtime(srcp)] + [os.path.getmtime(d) for d in _deps()])
    if os.path.exists(obj) and os.path.getmtime(obj) >= newest and not _foreign(obj):
        return obj
    cmd = [nvcc()] + ARCH + NVCC_FLAGS + extra + ["-c", srcp, "-o", obj]
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{proc.stdout}\n{proc.stderr}")
    return obj


_ELF_MACHINES = {"x86_64": 62, "AMD64": 62, "aarch64": 183, "arm64": 183}


def _elf_machine(path: str) -> int | None:
    """e_machine of an ELF file (None if unreadable)."""
    try:
        with open(path, "rb") as fp:
            head = fp.read(20)
    except OSError:
        return None
    if len(head) < 20 or head[:4] != b"\x7fELF":
        return None
    return struct.unpack_from("<H", head, 18)[0]


def _foreign(path: str) -> bool:
    """True when `path` exists but was built for another machine than this one."""
    want = _ELF_MACHINES.get(platform.machine())
    return os.path.exists(path) and want is not None and _elf_machine(path) != want


def build(verbose: bool = False, extra: list[str] | None = None) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    os.makedirs(OBJ_DIR, exist_ok=True)
    extra = extra or []
    srcs = [s for s in SOURCES if os.path.exists(os.path.join(CSRC, s))]
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra), srcs))
    if (not os.path.exists(LIB) or _foreign(LIB) or
            os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs)):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"]
        proc = subprocess.run(cmd, capture_output=True, text=True)
        if proc.returncode != 0:
            raise RuntimeError(f"link failed:\n{proc.stdout}\n{proc.stderr}")
    if verbose:
        print(LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True, extra=sys.argv[1:])
