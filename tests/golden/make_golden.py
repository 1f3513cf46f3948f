"""Generate the golden vectors of the reference CPU path (run in the build
container, where the reference tree exists; the fixtures are committed).

The reference's own solver (FDTD_CPU.cxx + FDTD_common.cxx, compiled
unchanged by oracle/build.py with the one-token fix of FDTD_CPU.cxx:816 done by
the compiler) is driven by oracle/ref_driver.cpp:

* ``fitness`` mode: the full entry point FDTD_CPU(args) at the reference's
  compile-time size (401x401, 2000 steps, 4 plane waves);
* ``steps`` mode: the same functions for STEPS time steps per excitation,
  dumping Ez probe traces, far-field magnitudes D, the running-DFT surface
  currents and the final fields of excitation 0.

Inputs: vacuum, a uniform dielectric (eps_r = 4, sigma = 0.05 S/m) and a
seeded random 9x9 patch image (tomography_gb300.workloads.reference_patch_args).

The far-field targets the reference compiles in (FDTD_CPU.cxx:789, 4000
values; FDTD_GPU.cu:996, 8000 values of which the first 4000 are magnitudes)
are parsed out of the reference sources into ref_measurement_{cpu,gpu}.npy so
that the drop-in FDTD_GPU can be given its target as data.

Usage:  python tests/golden/make_golden.py [--steps 1000] [--skip-full]
"""
from __future__ import annotations

import argparse
import os
import struct
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(REPO, "oracle"))

import build as oracle_build  # noqa: E402
from tomography_gb300.workloads import reference_patch_args  # noqa: E402

CASES = {
    "vacuum": lambda: np.array([1.0] * 81 + [0.0] * 81),
    "dielectric": lambda: np.array([4.0] * 81 + [0.05] * 81),
    "random": lambda: reference_patch_args(0x70F00000 + 77, cpu_variant=True),
}
ACC_FREQS = [0, 4, 9]
WIN = (168, 232)   # 64x64 window over the breast (cells 168..231)


def read_dump(path: str) -> dict:
    out = {}
    with open(path, "rb") as fp:
        data = fp.read()
    off = 0
    while off < len(data):
        (nl,) = struct.unpack_from("<I", data, off); off += 4
        name = data[off:off + nl].decode(); off += nl
        (nd,) = struct.unpack_from("<I", data, off); off += 4
        shape = struct.unpack_from("<" + "I" * nd, data, off); off += 4 * nd
        count = int(np.prod(shape))
        out[name] = np.frombuffer(data, dtype=np.float32, count=count, offset=off).reshape(shape).copy()
        off += 4 * count
    return out


def extract_measurement(path: str, line_no: int) -> np.ndarray:
    """The initializer list of `float measurement[...] = { ... };` on line line_no."""
    with open(path, errors="replace") as fp:
        line = fp.readlines()[line_no - 1]
    body = line[line.index("{") + 1: line.rindex("}")]
    return np.array([float(v) for v in body.split(",") if v.strip()], dtype=np.float32)


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--skip-full", action="store_true")
    ap.add_argument("--cases", default=",".join(CASES))
    opt = ap.parse_args()
    if not oracle_build.build_reference():
        sys.exit("reference tree not available")
    drv = oracle_build.ref_driver_path()
    tree = oracle_build.reference_source_dir()
    m_cpu = extract_measurement(os.path.join(tree, "FDTD_CPU.cxx"), 789)
    m_gpu = extract_measurement(os.path.join(tree, "FDTD_GPU.cu"), 996)
    np.save(os.path.join(HERE, "ref_measurement_cpu.npy"), m_cpu)
    np.save(os.path.join(HERE, "ref_measurement_gpu.npy"), m_gpu)
    print("measurement vectors:", m_cpu.shape, m_gpu.shape)
    with tempfile.TemporaryDirectory() as tmp:
        for name in opt.cases.split(","):
            args = CASES[name]()
            apath = os.path.join(tmp, name + ".txt")
            with open(apath, "w") as fp:
                fp.write("\n".join("%.17g" % v for v in args))
            rec = {"args": args, "steps": np.int32(opt.steps)}
            if not opt.skip_full:
                fpath = os.path.join(tmp, name + ".fit")
                subprocess.run([drv, "fitness", apath, fpath], check=True)
                rec["fitness_full"] = np.float64(open(fpath).read().strip())
            bpath = os.path.join(tmp, name + ".bin")
            subprocess.run([drv, "steps", apath, str(opt.steps), bpath], check=True)
            d = read_dump(bpath)
            rec["probe_xy"] = d["probe_xy"].astype(np.int32)
            rec["traces"] = d["traces"]
            rec["D"] = d["D"]
            if name != "vacuum":
                for k, v in d.items():
                    if k.startswith(("cj", "cm")):
                        rec[k] = v[ACC_FREQS]
                rec["acc_freqs"] = np.array(ACC_FREQS, dtype=np.int32)
                lo, hi = WIN
                rec["win"] = np.array(WIN, dtype=np.int32)
                rec["Ez_win"] = d["Ez_e0"][lo:hi, lo:hi]
                rec["Hx_win"] = d["Hx_e0"][lo:hi, lo:hi]
                rec["Hy_win"] = d["Hy_e0"][lo:hi, lo:hi]
                rec["Ez_sub8"] = d["Ez_e0"][::8, ::8]
                rec["Hy_sub8"] = d["Hy_e0"][::8, ::8]
            out = os.path.join(HERE, f"ref_cpu_{name}.npz")
            np.savez_compressed(out, **rec)
            print("wrote", out, os.path.getsize(out), "bytes")


if __name__ == "__main__":
    main()
