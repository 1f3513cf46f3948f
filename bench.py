"""Benchmark of the batched PSO fitness path (breast-imaging workload 1).

One step = one PSO generation: tomo_fitness_batch() over 256 candidates x 16
transmitters = 4096 forward solves on a 400x400 grid (12-cell CPML, 3000
steps, FP32 fields), seeded synthetic candidates and target, through the C ABI.

  value : evals/s from device time (CUDA events on the library's launching
          stream around set-up + time loop + far field + misfit; inputs resident)
  e2e   : evals/s of the same C-ABI call timed on the host with host buffers
          (H2D of the candidate parameters, D2H of the fitness inside)
  roofline : the advance kernel, algorithmic 48 B per FP32 cell-update
  cpu_baseline : the oracle's FP32 port of the reference CPU solver, one
          candidate (16 solves) on all host cores

python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
Under torchrun each rank evaluates its own generation (replicas, weak scaling).
"""
from __future__ import annotations

import argparse
import json
import os
import re
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

METRIC = "PSO fitness evals/s"
CONFIG_INDEX = 1
N_CAND = 256
BYTES_PER_CELL_UPDATE = 48.0   # FP32: Ez, Hx, Hy, Jp read+write + 4 per-cell coefficients


def _rank_info():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def _peaks() -> dict:
    path = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as fp:
            d = json.load(fp)
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


def _profile_traffic() -> float | None:
    """DRAM bytes per cell-update of the advance kernel from the committed ncu summary."""
    path = os.path.join(REPO, "profiles", "fdtd_advance_pso400.txt")
    if not os.path.exists(path):
        return None
    for line in open(path):
        m = re.match(r"\s*dram_bytes_per_cell_update:\s*([0-9.eE+-]+)", line)
        if m:
            return float(m.group(1))
    return None


class ClockSampler:
    """nvidia-smi clock / throttle-reason sampling during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.rows = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 7:
                self.rows.append(parts)

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=5)
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if r[3 + i].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def cpu_baseline_sample(spec_dict: dict, params: np.ndarray, threads: int) -> tuple[float, dict]:
    """Oracle FP32 port of the reference CPU solver: one candidate = n_tx solves,
    one per host thread.  Returns (evals/s, description)."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import model as M  # the oracle (checker / baseline leg only)

    probs = [M.breast_problem(spec_dict, params, t) for t in range(spec_dict["n_tx"])]
    t0 = time.perf_counter()
    M.run(probs, bits=32, threads=threads)
    dt = time.perf_counter() - t0
    return 1.0 / dt, {"seconds": dt, "solves": len(probs)}


def run_reference(args) -> None:
    rank, world, _ = _rank_info()
    if rank != 0:
        return
    import tomography_gb300 as T
    from tomography_gb300 import workloads as W

    spec = T.breast_spec(CONFIG_INDEX).as_dict()
    cand = W.candidate_batch(CONFIG_INDEX, 1, spec["n_ellipses"])[0]
    threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        cpu_baseline_sample(spec, cand, threads)
    vals = []
    t0 = time.perf_counter()
    for _ in range(args.steps):
        v, _ = cpu_baseline_sample(spec, cand, threads)
        vals.append(v)
    wall = time.perf_counter() - t0
    value = args.steps / wall
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "evals/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * wall / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded candidates)",
        "config": {"workload": "breast-imaging PSO generation: 400x400, 12-cell CPML, 3000 steps, 16 tx/candidate, "
                               "8 ellipses (64 params); reference arm = 1 candidate per step",
                   "grid": 400, "steps_per_solve": 3000, "tx_per_candidate": 16, "parallelism": "host threads"},
        "cpu_baseline": {"value": value, "unit": "evals/s", "cores": threads, "kind": "port",
                         "sample": "1 candidate (16 transmitter solves, 400x400 x 3000 steps) per step, "
                                   "one solve per host thread, oracle FP32 port of FDTD_CPU.cxx"},
        "e2e": {"value": value, "unit": "evals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_ours(args) -> None:
    rank, world, local = _rank_info()
    import torch

    dist = None
    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)
    dev = torch.device("cuda", torch.cuda.current_device())

    import tomography_gb300 as T
    from tomography_gb300 import workloads as W

    spec = T.breast_spec(CONFIG_INDEX)
    ncand = args.candidates
    K = spec.n_ellipses
    # candidates of this rank (replicas: each rank its own generation)
    cands = W.candidate_batch(CONFIG_INDEX, ncand * world, K)[rank * ncand:(rank + 1) * ncand]
    cands = np.ascontiguousarray(cands)
    fit = np.zeros(ncand, dtype=np.float64)

    # target: traces of the seeded target phantom (3 fibroglandular ellipses)
    tspec = spec.copy(n_ellipses=3)
    with T.Solver(tspec) as ts:
        target = ts.forward(W.target_phantom(CONFIG_INDEX, 3), traces=True, far_field=False)["traces"][0]
    solver = T.Solver(spec)
    solver.set_target(target)

    def barrier():
        torch.cuda.synchronize(dev)
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize(dev)

    for _ in range(args.warmup):
        solver.fitness_batch(cands, out=fit)
    stats0 = solver.stats()

    sampler = ClockSampler(dev.index if dev.index is not None else 0)
    sampler.start()
    barrier()
    dev_ms, adv_ms, wall = [], [], []
    kernels = 0
    t_start = time.perf_counter()
    for _ in range(args.steps):
        t0 = time.perf_counter()
        solver.fitness_batch(cands, out=fit)
        wall.append(time.perf_counter() - t0)
        st = solver.stats()
        dev_ms.append(st["total_ms"])
        adv_ms.append(st["advance_ms"])
        kernels += st["kernels"]
    barrier()
    elapsed = time.perf_counter() - t_start
    clocks = sampler.stop()
    st = solver.stats()

    # max over ranks of the device and host times
    tot_dev = sum(dev_ms) / 1e3
    tot_wall = sum(wall)
    if dist is not None:
        t = torch.tensor([tot_dev, tot_wall, elapsed], device=dev, dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        tot_dev, tot_wall, elapsed = t.tolist()
    units = ncand * world * args.steps
    value = units / tot_dev
    e2e = units / tot_wall

    # roofline of the advance kernel (average launch over the timed region)
    launches = st["launches"]
    cells_per_launch = st["cell_updates"] / launches   # solves * nx * ny * T (average over launches)
    launch_s = (sum(adv_ms) / len(adv_ms)) / 1e3 / launches
    achieved = BYTES_PER_CELL_UPDATE * cells_per_launch / launch_s / 1e9
    peaks = _peaks()
    tr = _profile_traffic()
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                "frac": achieved / peaks["hbm_gbs"], "peak_source": peaks["source"],
                "traffic": (tr * cells_per_launch) if tr is not None else None,
                "algorithmic_bytes_per_launch": BYTES_PER_CELL_UPDATE * cells_per_launch,
                "kernel": "fdtd_advance_kernel<float,%d,%d>" % (st["steps_per_launch"], st["cols_per_lane"])}
    gcells = st["cell_updates"] * world * args.steps / tot_dev / 1e9

    extra = {}
    if rank == 0 and world == 1 and not args.no_extras:
        # FP64 plain path (one solve per launch sequence, one launch per step, no graph):
        # the denominator of the batching + precision speed-up, timed on one candidate
        pspec = spec.copy(precision=T.FP64, steps_per_launch=1, cols_per_lane=1, plain=1)
        with T.Solver(pspec) as ps:
            ps.set_target(target)
            ps.fitness(cands[0])   # warm-up
            t0 = time.perf_counter()
            out64 = ps.forward(cands[:1], traces=False, traces_f64=True, far_field=False, fitness=True)
            plain_s = time.perf_counter() - t0
        out32 = solver.forward(cands[:1], traces=True, far_field=False, fitness=True)
        tr64 = out64["traces_f64"][0]
        err = float(np.linalg.norm(out32["traces"][0].astype(np.float64) - tr64) / np.linalg.norm(tr64))
        ferr = float(abs(out32["fitness"][0] - out64["fitness"][0]) / abs(out64["fitness"][0]))
        extra["fp64_plain"] = {"evals_per_s": 1.0 / plain_s, "speedup_of_value": value / (1.0 / plain_s)}
        extra["error_vs_fp64"] = {"trace_rel_l2": err, "fitness_rel": ferr, "candidates": 1}
        extra["fitness_head"] = [float(v) for v in fit[:4]]
        # reported CPU baseline: oracle FP32 port of the reference CPU solver
        threads = os.cpu_count() or 1
        cb, info = cpu_baseline_sample(spec.as_dict(), cands[0], threads)
        extra["cpu_baseline"] = {"value": cb, "unit": "evals/s", "cores": threads, "kind": "port",
                                 "sample": "1 candidate = 16 transmitter solves (400x400 x 3000 steps), one per "
                                           "host thread, oracle FP32 port of FDTD_CPU.cxx (%.1f s)" % info["seconds"]}

    lat = sorted(w * 1e3 for w in wall)
    line = {
        "metric": METRIC, "value": value, "unit": "evals/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * tot_dev / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded candidates and target phantom)",
        "config": {"workload": "breast-imaging PSO generation (batched fitness)", "grid": 400, "dx_mm": 0.5,
                   "cpml_cells": 12, "steps_per_solve": spec.steps, "candidates_per_gpu": ncand,
                   "tx_per_candidate": spec.n_tx, "solves_per_step": ncand * spec.n_tx, "params_per_candidate": 64,
                   "parallelism": f"replicas x{world}", "l2": "inputs larger than L2 (%.0f GB state)" % (
                       ncand * spec.n_tx * 400 * 400 * 4 * 8 / 1e9),
                   "steps_per_launch": st["steps_per_launch"], "cols_per_lane": st["cols_per_lane"]},
        "e2e": {"value": e2e, "unit": "evals/s", "h2d_bytes_per_step": int(st["h2d_bytes"]),
                "d2h_bytes_per_step": int(st["d2h_bytes"])},
        "gcell_updates_per_s": gcells,
        "latency_ms": {"p50": lat[len(lat) // 2], "p99": lat[min(len(lat) - 1, int(0.99 * len(lat)))],
                       "per": "generation of %d evaluations" % ncand},
        "roofline": roofline,
        "clocks": clocks,
        "gpu_launches": int(kernels),
    }
    line.update(extra)
    if "cpu_baseline" not in line:
        line["cpu_baseline"] = None
    if rank == 0:
        print(json.dumps(line), flush=True)
    solver.close()
    if dist is not None:
        dist.destroy_process_group()


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--candidates", type=int, default=N_CAND)
    ap.add_argument("--no-extras", action="store_true")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
