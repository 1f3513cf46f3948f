"""The C++ drop-in, called the way the reference's search binds it.

A small C++ program includes ``tomography_fdtd.hpp``, takes ``FDTD_GPU`` as a
``double (*)(const std::vector<double>&)`` -- the function-pointer type
tao's ``ps.go(FDTD_GPU)`` receives (test.cxx:94-121) -- and links the
library.  The target is read from TOMO_MEASUREMENT_FILE, as raw float32, as
text, and as the reference's whole 8000-entry array (of which its misfit uses
the first 4000).  Two calls in a row must give exactly the fitness of the batch API
for the same arguments, and a short argument vector must throw
std::out_of_range (the reference's ``.at()``).
"""
from __future__ import annotations

import os
import shutil
import subprocess

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROGRAM = r"""
#include "tomography_fdtd.hpp"
#include <cstdio>
#include <cstdlib>
#include <stdexcept>
#include <vector>

int main(int argc, char** argv) {
    std::vector<double> args;
    for (int i = 1; i < argc; ++i) args.push_back(std::strtod(argv[i], nullptr));
    double (*fitness)(const std::vector<double>&) = FDTD_GPU;
    const double f1 = fitness(args);
    const double f2 = fitness(args);
    std::printf("%.17g %.17g\n", f1, f2);
    try {
        fitness(std::vector<double>(args.begin(), args.begin() + 20));
        std::printf("no exception\n");
        return 1;
    } catch (const std::out_of_range&) {
        std::printf("out_of_range\n");
    }
    tomo_fdtd_gpu_release();
    return 0;
}
"""


def _build(tomo, tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    lib_dir = os.path.dirname(tomo.LIB_PATH)
    src = tmp_path / "dropin.cpp"
    src.write_text(PROGRAM)
    exe = tmp_path / "dropin"
    subprocess.run([cxx, "-std=c++17", "-O1", "-I", os.path.join(REPO, "include"), str(src), "-o", str(exe),
                    "-L", lib_dir, "-ltomography_gb300", "-Wl,-rpath," + lib_dir], check=True)
    return exe


def test_cpp_caller_compiles_and_links(tomo, tmp_path):
    """CPU: the reference-side C++ caller builds against the header and library."""
    assert _build(tomo, tmp_path).exists()


@pytest.mark.gpu
def test_cpp_dropin_matches_batch_api(tomo, tmp_path):
    from tomography_gb300 import workloads as W

    exe = _build(tomo, tmp_path)
    meas = np.load(os.path.join(REPO, "tests", "golden", "ref_measurement_gpu.npy"))[:4000].astype(np.float32)
    args = W.reference_patch_args(11)
    with tomo.Solver(tomo.reference_spec(False)) as s:
        s.set_target(meas)
        want = s.fitness(args)
    raw = tmp_path / "measurement.f32"
    meas.tofile(raw)
    txt = tmp_path / "measurement.txt"
    txt.write_text("\n".join(repr(float(v)) for v in meas))
    full = tmp_path / "measurement8000.f32"   # the reference's whole 8000-entry array: first 4000 used
    np.load(os.path.join(REPO, "tests", "golden", "ref_measurement_gpu.npy")).astype(np.float32).tofile(full)
    for path in (raw, txt, full):
        env = dict(os.environ, TOMO_MEASUREMENT_FILE=str(path))
        out = subprocess.run([str(exe)] + [repr(float(a)) for a in args], env=env, capture_output=True, text=True,
                             timeout=600)
        assert out.returncode == 0, out.stdout + out.stderr
        lines = out.stdout.split()
        f1, f2 = float(lines[0]), float(lines[1])
        assert f1 == want and f2 == want, (path.name, f1, f2, want)
        assert lines[2] == "out_of_range"
