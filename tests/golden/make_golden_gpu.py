"""Generate the golden vectors of the reference GPU path (run on the GPU host;
the fixtures it writes are committed under tests/golden/).

The reference's own GPU solver (FDTD_GPU.cu + FDTD_common.cxx, compiled
unchanged for sm_103a by oracle/build.py::build_reference_gpu, from the
reference tree or its staged copy under oracle/_ref/src/) is driven by
oracle/ref_gpu_driver.cpp: the full entry point FDTD_GPU(args) at the
reference's compile-time size (401x401, 2000 steps, 4 plane waves, 10
frequencies, 100 angles), its fitness against the target it compiles in
(FDTD_GPU.cu:996), its running-DFT surface currents and the far field D / P
recomputed from them by its own N2FPostProcess.

Inputs (27 arguments: 3x3 patches of eps_inf, then del_eps, then sigma):
  vacuum  eps_inf 1, del_eps 0, sigma 0 (no scatterer: D == 0)
  hinted  the phantom of the reference's commented-out defaults
          (FDTD_GPU.cu:659-692): fat (eps_inf 3.14, del_eps 1.61) with
          eps_inf 6.75, del_eps 40 in patch numpatches/2, sigma 0
  random  a seeded draw within the reference's search bounds
          (tomography_gb300.workloads.reference_patch_args)

Each case calls FDTD_GPU `--reps` times; the wall time of every call is kept
(the first includes CUDA context and module set-up).

Usage:  python tests/golden/make_golden_gpu.py [--out DIR] [--reps 3] [--cases vacuum,hinted,random]
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(REPO, "oracle"))
sys.path.insert(0, HERE)

import build as oracle_build  # noqa: E402
from make_golden import read_dump  # noqa: E402
from tomography_gb300.workloads import reference_patch_args  # noqa: E402


def hinted_args() -> np.ndarray:
    einf = [3.14] * 9
    deps = [1.61] * 9
    einf[1], deps[1] = 6.75, 40.0   # patch numpatches/2 = 1
    return np.array(einf + deps + [0.0] * 9, dtype=np.float64)


CASES = {
    "vacuum": lambda: np.array([1.0] * 9 + [0.0] * 18, dtype=np.float64),
    "hinted": hinted_args,
    "random": lambda: reference_patch_args(0x70F00000 + 91),
}
FAMILIES = ("cjzyn", "cjzxp", "cjzyp", "cjzxn", "cmxyn", "cmyxp", "cmxyp", "cmyxn")


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=HERE)
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--cases", default=",".join(CASES))
    args = ap.parse_args()
    if not oracle_build.build_reference_gpu():
        sys.exit("reference GPU sources or nvcc unavailable")
    drv = oracle_build.ref_gpu_driver_path()
    os.makedirs(args.out, exist_ok=True)
    with tempfile.TemporaryDirectory() as tmp:
        for case in args.cases.split(","):
            a = CASES[case]()
            apath = os.path.join(tmp, f"{case}.txt")
            np.savetxt(apath, a, fmt="%.17g")
            bpath = os.path.join(tmp, f"{case}.bin")
            proc = subprocess.run([drv, "run", apath, bpath, str(args.reps)], capture_output=True, text=True)
            if proc.returncode != 0:
                sys.stderr.write(proc.stdout[-2000:] + proc.stderr[-2000:])
                sys.exit(f"reference GPU driver failed for {case} (rc {proc.returncode})")
            dump = read_dump(bpath)
            rec = {"args": a, "D": dump["D"], "P": dump["P"], "fitness": np.float64(dump["fitness"][-1]),
                   "fitness_calls": dump["fitness"].astype(np.float64), "seconds": dump["seconds"].astype(np.float64)}
            for fam in FAMILIES:
                rec[fam] = dump[fam]
            np.savez_compressed(os.path.join(args.out, f"ref_gpu_{case}.npz"), **rec)
            print(json.dumps({"case": case, "fitness": float(rec["fitness"]),
                              "seconds_per_call": [float(s) for s in rec["seconds"]],
                              "max_D": float(np.abs(rec["D"]).max())}), flush=True)


if __name__ == "__main__":
    main()
