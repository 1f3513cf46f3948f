"""CPU: the C-ABI library loads, exports every declared symbol, and its host
logic (presets, validation, error reporting) works without a GPU."""
from __future__ import annotations

import ctypes as C
import os
import re

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared_functions() -> list[str]:
    names = set()
    for fn in os.listdir(os.path.join(REPO, "include")):
        # tomography_search.hpp is header-only C++ over the C ABI (its own test
        # compiles a caller); the other headers declare library symbols
        if fn == "tomography_search.hpp":
            continue
        text = open(os.path.join(REPO, "include", fn)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        text = re.sub(r"//[^\n]*", "", text)
        text = re.sub(r"typedef\s+[^;{}]*\(\s*\*[^;{}]*;", "", text)   # function-pointer types
        for m in re.finditer(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\([^;{}]*\)\s*;", text):
            name = m.group(1)
            if name not in ("if", "while", "for", "sizeof", "return"):
                names.add(name)
    return sorted(names)


def test_library_exports_every_declared_symbol(tomo):
    lib = tomo.library()
    declared = _declared_functions()
    assert "tomo_fitness_batch" in declared and "FDTD_GPU" in declared
    for name in declared:
        if name == "FDTD_GPU":
            # C++ linkage: double FDTD_GPU(const std::vector<double>&)
            getattr(lib, "_Z8FDTD_GPURKSt6vectorIdSaIdEE")
        else:
            getattr(lib, name)


def test_presets(tomo):
    r = tomo.reference_spec(False)
    assert (r.nx, r.ny, r.steps, r.ncpml, r.nfreq, r.n_angles, r.nf2ff_d) == (401, 401, 2000, 10, 10, 100, 100)
    assert r.npatch == 3 and r.misfit == 0 and r.pw_centred == 1
    c = tomo.reference_spec(True)
    assert c.npatch == 9 and c.misfit == 1 and c.pw_centred == 0
    b = tomo.breast_spec(1)
    assert (b.nx, b.steps, b.ncpml, b.n_tx, b.n_ellipses) == (400, 3000, 12, 16, 8)
    assert b.dt == pytest.approx(0.99 * 0.5e-3 / (299792458.0 * np.sqrt(2)), rel=1e-4)
    lib = tomo.library()
    assert lib.tomo_num_params(C.byref(r)) == 27
    assert lib.tomo_num_params(C.byref(c)) == 162
    assert lib.tomo_num_params(C.byref(b)) == 64
    assert lib.tomo_num_excitations(C.byref(b)) == 16
    assert lib.tomo_spec_breast(C.byref(b), 9) == -1
    assert b"0..4" in lib.tomo_last_error()
    # serving requests: the disc stays at 70% of a 100 mm domain, steps = 4 x edge
    for edge, ant in ((128, 8), (1024, 32)):
        v = tomo.serving_spec(edge, ant)
        assert (v.nx, v.ny, v.steps, v.n_antennas, v.n_tx) == (edge, edge, 4 * edge, ant, ant)
        assert v.dx == pytest.approx(0.1 / edge) and 2 * v.disc_radius / (v.nx * v.dx) == pytest.approx(0.7)
        assert v.dt == pytest.approx(0.99 * v.dx / (299792458.0 * np.sqrt(2)), rel=1e-4)
        assert v.cpml_sigma_max == pytest.approx(0.8 * 4 / (376.730313 * v.dx), rel=1e-6)
    assert lib.tomo_spec_serving(C.byref(b), 32, 8) == -1


def test_invalid_specs_are_rejected_before_device_use(tomo):
    lib = tomo.library()
    bad = [
        tomo.breast_spec(0).copy(nx=4),
        tomo.breast_spec(0).copy(steps=0),
        tomo.breast_spec(0).copy(ncpml=200),
        tomo.breast_spec(0).copy(n_antennas=0),
        tomo.breast_spec(0).copy(n_tx=99),
        tomo.breast_spec(0).copy(antenna_radius=1.0),
        tomo.reference_spec(False).copy(ny=300),
        tomo.breast_spec(0).copy(precision=7),
        # the total-field variant belongs to the reference GPU mode only
        tomo.breast_spec(0).copy(total_field=1),
        tomo.reference_spec(True).copy(total_field=1),
        tomo.reference_spec(False).copy(total_field=2),
    ]
    for s in bad:
        h = C.c_void_p()
        rc = lib.tomo_create(C.byref(s), C.byref(h))
        assert rc == -1, (rc, lib.tomo_last_error())
        assert not h.value


def test_no_cpu_fallback_without_gpu(tomo):
    """On a host without a GPU the product refuses to run instead of falling back."""
    import torch

    if torch.cuda.is_available():
        pytest.skip("GPU present")
    with pytest.raises(tomo.TomoError) as ei:
        tomo.Solver(tomo.breast_spec(0))
    assert ei.value.status == -5


def test_workload_generator_is_deterministic():
    from tomography_gb300 import workloads as W

    g = W.SplitMix64(0)
    # published splitmix64 sequence for seed 0
    assert g.next_u64() == 0xE220A8397B1DCDAF
    assert g.next_u64() == 0x6E789E6AA1B965F4
    a = W.candidate_batch(1, 3, 8)
    b = W.candidate_batch(1, 3, 8)
    assert a.shape == (3, 64) and np.array_equal(a, b)
    t = W.target_phantom(1)
    assert t.shape == (24,) and np.all(t[5::8] == 12.9)


def test_save_field_image(tomo, tmp_path):
    f = np.linspace(-1, 1, 12, dtype=np.float32).reshape(3, 4)
    tomo.save_field(str(tmp_path / "f.npy"), f)
    np.testing.assert_array_equal(np.load(tmp_path / "f.npy"), f)
    tomo.save_field(str(tmp_path / "f.pgm"), f)
    data = (tmp_path / "f.pgm").read_bytes()
    assert data.startswith(b"P5\n4 3\n255\n") and len(data) == len(b"P5\n4 3\n255\n") + 12
    img = np.frombuffer(data[-12:], dtype=np.uint8).reshape(3, 4)
    assert img[-1, 0] == 0 and img[0, -1] == 255   # rows stored top (largest y) first
    with pytest.raises(ValueError):
        tomo.save_field(str(tmp_path / "f.png"), f)


def test_dropin_target_file_rules(tomo, tmp_path):
    """TOMO_MEASUREMENT_FILE parsing of the drop-in (no GPU needed): raw float32
    or text, 4000 values or the reference's 8000 (first 4000 used); a .npy file,
    text with other content, or another length is refused."""
    meas = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_measurement_gpu.npy"))
    meas = meas.astype(np.float32)
    assert meas.size == 8000
    raw = tmp_path / "m.f32"
    meas.tofile(raw)
    np.testing.assert_array_equal(tomo.read_target_file(str(raw)), meas[:4000])
    meas[:4000].tofile(raw)
    np.testing.assert_array_equal(tomo.read_target_file(str(raw)), meas[:4000])
    txt = tmp_path / "m.txt"
    txt.write_bytes(b"\xef\xbb\xbf" + ", ".join("%.9g" % v for v in meas[:4000]).encode() + b"\n")
    np.testing.assert_array_equal(tomo.read_target_file(str(txt)), meas[:4000])
    bad = {
        "npy": None,
        "comment": b"# magnitudes\n" + b" ".join(b"%.9g" % v for v in meas[:4000]),
        "c_literal": b"float measurement[] = {" + b",".join(b"%.9g" % v for v in meas[:4000]) + b"};",
        "short": meas[:3999].tobytes(),
        "odd_length": meas[:5000].tobytes(),
        "ragged_bytes": meas[:4000].tobytes() + b"\x01",
    }
    for name, data in bad.items():
        path = tmp_path / f"bad_{name}"
        if name == "npy":
            path = tmp_path / "m.npy"
            np.save(path, meas[:4000])
        else:
            path.write_bytes(data)
        with pytest.raises(tomo.TomoError) as ei:
            tomo.read_target_file(str(path))
        assert ei.value.status == -1, name
    with pytest.raises(tomo.TomoError):
        tomo._target_values(meas[:5000])


C_PROGRAM = r"""
#include "tomography.h"
#include <stdio.h>
static int bowl(void *user, const double *pop, size_t n, size_t np, double *fit) {
    (void)user;
    for (size_t i = 0; i < n; ++i) {
        double s = 0;
        for (size_t j = 0; j < np; ++j) { double d = pop[i * np + j] - 0.25; s += d * d; }
        fit[i] = -s;
    }
    return TOMO_OK;
}
int main(void) {
    tomo_spec s;
    if (tomo_spec_breast(&s, 1) != TOMO_OK) return 1;
    tomo_search_params p;
    const char *argv[] = {"--population_size", "20", "--maximum_iterations", "60", "--seed", "3"};
    if (tomo_search_defaults(&p, TOMO_SEARCH_DE) || tomo_search_parse_args(&p, 6, argv)) return 2;
    double lo[4] = {-1, -1, -1, -1}, hi[4] = {1, 1, 1, 1}, best[4], fit;
    int64_t evals = 0;
    int rc = tomo_search_run(&p, lo, hi, 4, bowl, NULL, NULL, NULL, best, &fit, NULL, &evals);
    printf("%d %d %lld %.17g\n", tomo_num_params(&s), rc, (long long)evals, fit);
    return rc;
}
"""


def test_c_header_is_c99_and_links(tomo, tmp_path):
    """include/tomography.h is a C header (strict C99, no warnings), and a C
    caller links the library and runs a search through it with a C callback;
    the tao-style C++ caller of the drop-in (a double (*)(const
    std::vector<double>&) bound to FDTD_GPU) compiles and links."""
    import shutil
    import subprocess

    cc, cxx = shutil.which("gcc") or shutil.which("cc"), shutil.which("g++") or shutil.which("c++")
    if cc is None or cxx is None:
        pytest.skip("no C/C++ compiler")
    lib_dir = os.path.dirname(tomo.LIB_PATH)
    inc = os.path.join(REPO, "include")
    link = ["-L", lib_dir, "-ltomography_gb300", "-Wl,-rpath," + lib_dir]
    src = tmp_path / "caller.c"
    src.write_text(C_PROGRAM)
    exe = tmp_path / "caller"
    subprocess.run([cc, "-std=c99", "-Wall", "-Wextra", "-Werror", "-pedantic", "-I", inc, str(src), "-o", str(exe)]
                   + link, check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()
    assert out[:3] == ["64", "0", str(20 * 61)] and float(out[3]) > -1e-6
    cpp = tmp_path / "dropin.cpp"
    cpp.write_text('#include "tomography_fdtd.hpp"\n#include <vector>\n'
                   'int main() { double (*f)(const std::vector<double>&) = FDTD_GPU; return f == nullptr; }\n')
    subprocess.run([cxx, "-std=c++17", "-Wall", "-Werror", "-I", inc, str(cpp), "-o", str(tmp_path / "dropin")]
                   + link, check=True)


def test_python_signatures_match_the_c_header(tomo):
    """The ctypes binding declares each C function with as many arguments as
    include/tomography.h and the drop-in header give it, and a void return
    exactly where the header has one."""
    text = ""
    for fn in ("tomography.h", "tomography_fdtd.hpp"):
        text += open(os.path.join(REPO, "include", fn)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    text = re.sub(r"//[^\n]*", "", text)
    text = re.sub(r"typedef\s+[^;{}]*\(\s*\*[^;{}]*;", "", text)
    protos = {}
    for m in re.finditer(r"\b(int|void|const char\s*\*)\s*(tomo_\w+)\s*\(([^;{}]*)\)\s*;", text):
        params = m.group(3).strip()
        n = 0 if params in ("", "void") else params.count(",") + 1
        protos[m.group(2)] = (m.group(1).strip(), n)
    lib = tomo.library()
    checked = 0
    for name, (ret, n) in protos.items():
        fn = getattr(lib, name)
        if fn.argtypes is None:
            continue                                  # not bound in Python
        assert len(fn.argtypes) == n, (name, len(fn.argtypes), n)
        assert (fn.restype is None) == (ret == "void"), name
        checked += 1
    assert checked >= 30 and "tomo_search_run" in protos and "tomo_wait" in protos


def test_ctypes_structs_match_the_c_layout(tomo, tmp_path):
    """Every ctypes mirror of a C struct (tomo_spec, tomo_outputs, tomo_stats,
    tomo_search_params) has the C struct's size and each field at the C
    offset: a C program compiled against include/tomography.h prints
    sizeof/offsetof for the fields the mirrors name."""
    import shutil
    import subprocess

    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    from tomography_gb300.spec import Spec

    mirrors = {"tomo_spec": Spec, "tomo_outputs": tomo.Outputs, "tomo_stats": tomo.Stats,
               "tomo_search_params": tomo.SearchParams}
    lines = ['#include "tomography.h"', "#include <stddef.h>", "#include <stdio.h>", "int main(void) {"]
    for cname, py in mirrors.items():
        lines.append(f'    printf("{cname} size %zu\\n", sizeof({cname}));')
        for f in py._fields_:
            lines.append(f'    printf("{cname} {f[0]} %zu\\n", offsetof({cname}, {f[0]}));')
    lines += ["    return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-std=c99", "-I", os.path.join(REPO, "include"), str(src), "-o", str(exe)], check=True)
    got = {}
    for line in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.splitlines():
        cname, field, value = line.split()
        got[(cname, field)] = int(value)
    for cname, py in mirrors.items():
        assert C.sizeof(py) == got[(cname, "size")], cname
        for f in py._fields_:
            assert getattr(py, f[0]).offset == got[(cname, f[0])], (cname, f[0])


def test_target_files(tomo, tmp_path):
    """Targets round-trip through every save_target format (.npy, text, raw
    float32) in the shape set_target takes; a file of the wrong length, with
    non-numeric text, of a partial float32 or with non-finite values is
    refused; a reference-mode file may hold the reference's whole array
    (magnitudes then phases), of which the first half is the target."""
    rng = np.random.default_rng(3)
    spec = tomo.breast_spec(0).copy(n_tx=2, n_antennas=4, steps=50)
    t = rng.standard_normal(tomo.target_shape(spec)).astype(np.float32)
    for name in ("t.npy", "t.txt", "t.csv", "t.f32"):
        path = str(tmp_path / name)
        tomo.save_target(path, t)
        got = tomo.load_target(path, spec)
        assert got.shape == (2, 4, 50) and got.dtype == np.float32
        np.testing.assert_array_equal(got, t)
    bad = tmp_path / "short.f32"
    t.ravel()[:-1].tofile(bad)
    with pytest.raises(ValueError, match="values"):
        tomo.load_target(str(bad), spec)
    (tmp_path / "junk.txt").write_text("1.0, 2.0\n# comment\n")
    with pytest.raises(ValueError):
        tomo.load_target(str(tmp_path / "junk.txt"), spec)
    (tmp_path / "odd.bin").write_bytes(b"\x00" * 10)
    with pytest.raises(ValueError, match="float32"):
        tomo.load_target(str(tmp_path / "odd.bin"), spec)
    nan = t.copy()
    nan[0, 0, 0] = np.nan
    tomo.save_target(str(tmp_path / "nan.npy"), nan)
    with pytest.raises(ValueError, match="non-finite"):
        tomo.load_target(str(tmp_path / "nan.npy"), spec)
    ref = tomo.reference_spec(False)
    whole = rng.random(8000).astype(np.float32)
    whole.tofile(tmp_path / "meas.f32")
    np.testing.assert_array_equal(tomo.load_target(str(tmp_path / "meas.f32"), ref).ravel(), whole[:4000])
