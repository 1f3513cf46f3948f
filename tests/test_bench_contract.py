"""CPU: the reference arm of bench.py keeps its output contract.

One JSON line with the run's metric and unit, "impl": "reference", a
cpu_baseline block describing the run and an e2e block without host-device
bytes; ranks other than 0 print nothing and exit 0.
"""
from __future__ import annotations

import json
import os
import subprocess
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _run(env_extra):
    env = dict(os.environ, **env_extra)
    return subprocess.run([sys.executable, os.path.join(REPO, "bench.py"), "--impl", "reference", "--steps", "1",
                           "--warmup", "0"], capture_output=True, text=True, env=env, timeout=600, cwd=REPO)


@pytest.fixture(scope="module")
def reference_run():
    """One run of the reference arm (rank 0, one step) in a fresh interpreter,
    shared by the tests below: its printed lines, and whether the product
    package was imported or its native library mapped into the process."""
    code = ("import sys; sys.argv = ['bench.py', '--impl', 'reference', '--steps', '1', '--warmup', '0'];"
            "sys.path.insert(0, %r); import bench; bench.main();"
            "maps = open('/proc/self/maps').read();"
            "print('PRODUCT', any(m.startswith('tomography_gb300') for m in sys.modules),"
            " 'libtomography_gb300' in maps)") % REPO
    env = {k: v for k, v in os.environ.items() if k not in ("RANK", "WORLD_SIZE", "LOCAL_RANK")}
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600, cwd=REPO, env=env)
    assert out.returncode == 0, out.stderr
    lines = [l for l in out.stdout.splitlines() if l.strip()]
    return [l for l in lines if not l.startswith("PRODUCT")], [l for l in lines if l.startswith("PRODUCT")]


def test_reference_arm_json_line(reference_run):
    lines, _ = reference_run
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["metric"] == "PSO fitness evals/s" and d["unit"] == "evals/s"
    assert d["value"] > 0 and d["steps"] == 1 and d["higher_is_better"] is True
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["kind"] == "port" and cb["cores"] >= 1 and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": "evals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert d["config"]["grid"] == 400 and d["config"]["steps_per_solve"] == 3000


def test_reference_arm_other_ranks_are_silent():
    out = _run({"RANK": "1", "WORLD_SIZE": "2", "LOCAL_RANK": "1"})
    assert out.returncode == 0 and out.stdout.strip() == ""


def test_reference_arm_does_not_load_the_product(reference_run):
    """The reference arm runs the checker only: the product package is never
    imported and its native library never mapped into the process."""
    _, tail = reference_run
    assert tail == ["PRODUCT False False"], tail


def test_both_arms_report_the_same_config(reference_run):
    sys.path.insert(0, REPO)
    import bench

    d = json.loads(reference_run[0][0])
    assert d["config"] == bench.workload_config(1, bench.N_CAND)


def test_profile_summary_covers_the_autotuned_blockings():
    """The roofline's DRAM traffic comes from the committed ncu summary; it holds
    a capture (with its per-cell-update DRAM bytes) for each blocking the
    autotuner picks between on the PSO generation, and none for others."""
    import bench

    t4 = bench._profile_traffic(4, 2, 2)
    t2 = bench._profile_traffic(2, 2, 3)
    assert t4 is not None and t2 is not None
    # deeper temporal blocking moves fewer DRAM bytes per cell-update, both far below 48 B
    assert 0 < t4 < t2 < bench.BYTES_PER_CELL_UPDATE
    assert bench._profile_traffic(3, 1, 3) is None
