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


def rank_candidates(config: int, ncand: int, world: int, rank: int, n_ellipses: int) -> np.ndarray:
    """This rank's generation: replicas evaluate disjoint slices of one seeded
    candidate stream (ncand per rank), so the job's work grows with the ranks."""
    from tomography_gb300 import workloads as W

    cands = W.candidate_batch(config, ncand * world, n_ellipses)[rank * ncand:(rank + 1) * ncand]
    return np.ascontiguousarray(cands)


def max_over_ranks(values, dist=None, device=None) -> list:
    """Element-wise maximum of per-rank timings (the job is as slow as its slowest rank)."""
    if dist is None:
        return list(values)
    import torch

    t = torch.tensor(list(values), dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return t.tolist()


def _peaks() -> dict:
    path = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as fp:
            d = json.load(fp)
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


def _profile_traffic(T: int, cols: int, minb: int) -> float | None:
    """DRAM bytes per cell-update of the advance kernel from the committed ncu
    summary, when it holds a capture with the same blocking (each capture's
    section opens with its `blocking:` line)."""
    path = os.path.join(REPO, "profiles", "fdtd_advance_pso400.txt")
    if not os.path.exists(path):
        return None
    found, blocking = {}, None
    for line in open(path):
        m = re.match(r"\s*blocking:\s*T=(\d+)\s+COLS=(\d+)\s+MINB=(\d+)", line)
        if m:
            blocking = tuple(int(v) for v in m.groups())
        m = re.match(r"\s*dram_bytes_per_cell_update:\s*([0-9.eE+-]+)", line)
        if m and blocking is not None:
            found[blocking] = float(m.group(1))
    return found.get((T, cols, minb))


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


def workload_config(world: int, ncand: int) -> dict:
    """The benchmarked workload (breast-imaging workload 1), identical in both arms."""
    return {"workload": "breast-imaging PSO generation (batched fitness)", "grid": 400, "dx_mm": 0.5,
            "cpml_cells": 12, "steps_per_solve": 3000, "candidates_per_gpu": ncand, "tx_per_candidate": 16,
            "solves_per_step": ncand * 16, "params_per_candidate": 64, "parallelism": f"replicas x{world}",
            "l2": "inputs larger than L2 (%.0f GB state)" % (ncand * 16 * 400 * 400 * 4 * 8 / 1e9)}


def run_reference(args) -> None:
    """Reference arm: the reference's CPU algorithm for this workload, timed on
    the host cores.  The reference's own FDTD_CPU.cxx only runs its compiled-in
    plane-wave problem, so the arm runs the oracle's FP32 port of it in the
    breast-imaging mode (checker-side spec and candidates; the product library
    is not loaded), one candidate per step, one solve per host thread.  The
    per-evaluation work (16 solves of 400 x 400 x 3000 steps) is that of one
    candidate of the GPU arm's generation."""
    rank, world, _ = _rank_info()
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import model as M  # the oracle (reference arm)

    spec = M.breast_spec(CONFIG_INDEX)
    cand = M.workload_candidates(CONFIG_INDEX, 1, spec["n_ellipses"])[0]
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
        "config": workload_config(world, args.candidates),
        "cpu_baseline": {"value": value, "unit": "evals/s", "cores": threads, "kind": "port",
                         "sample": "each step: 1 candidate of the generation (16 transmitter solves, 400x400 x 3000 "
                                   "steps; the same per-evaluation work as the GPU arm), one solve per host thread, "
                                   "oracle FP32 port of FDTD_CPU.cxx"},
        "e2e": {"value": value, "unit": "evals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_cpu_reference(args) -> None:
    """The reference's own CPU solver (FDTD_CPU.cxx, compiled unchanged from the
    reference sources or their staged copy) timed on the host cores at its
    compile-time problem (401 x 401, 2000 steps, 4 plane waves, 10 DFT
    frequencies): one excitation of --cpu-steps steps per copy, one copy on
    one core (latency) and one copy per core on every core (throughput, as
    the reference farms one evaluation per MPI rank), built without and with
    flush-to-zero (-ffast-math).  An evaluation is 4 excitations of 2000 steps."""
    rank, _, _ = _rank_info()
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import build as OB  # checker build recipes

    if not (OB.build_reference() and OB.build_reference(ftz=True)):
        print(json.dumps({"workload": "cpu-reference", "unavailable": "reference CPU sources not staged"}))
        return
    import tempfile

    cores = os.cpu_count() or 1
    steps = args.cpu_steps
    res = {}
    with tempfile.TemporaryDirectory() as tmp:
        apath = os.path.join(tmp, "args.txt")
        np.savetxt(apath, [4.0] * 81 + [0.05] * 81, fmt="%.17g")   # eps_r 4, sigma 0.05 S/m in the 9x9 patches
        for name, exe in (("no_ftz", OB.ref_driver_path()), ("ftz", OB.ref_driver_ftz_path())):
            for label, n in (("1_core", 1), ("all_cores", cores)):
                out = subprocess.run([exe, "bench", apath, str(steps), str(n)], capture_output=True, text=True,
                                     check=True).stdout
                sec = float(out.split()[1])
                evals = n / (4 * sec * 2000.0 / steps)
                res[f"{name}_{label}"] = {"seconds": sec, "copies": n, "evals_per_s": evals,
                                          "s_per_eval": n / evals,
                                          "mcell_updates_per_s": n * 401 * 401 * steps / sec / 1e6}
    print(json.dumps({"workload": "cpu-reference", "what": "reference FDTD_CPU.cxx time loop (H, E, 10-frequency "
                      "running DFT), 401x401, eps_r 4 / sigma 0.05 patches; eval = 4 excitations x 2000 steps",
                      "steps_timed_per_copy": steps, "cores": cores, "machine": os.uname().machine,
                      "results": res}), flush=True)


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
    cands = rank_candidates(CONFIG_INDEX, ncand, world, rank, K)
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

    tune = None
    for w in range(args.warmup):
        solver.fitness_batch(cands, out=fit)
        if w == 0:
            st0 = solver.stats()
            tune = {"steps_per_launch": st0["steps_per_launch"], "cols_per_lane": st0["cols_per_lane"],
                    "min_blocks_per_sm": st0.get("min_blocks_per_sm"), "blockings_timed": st0["tuned_configs"],
                    "tune_ms": st0["tune_ms"]}

    sampler = ClockSampler(dev.index if dev.index is not None else 0)
    sampler.start()
    barrier()
    torch.cuda.nvtx.range_push("timed")   # lets a profiler select the timed generations
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
    torch.cuda.nvtx.range_pop()
    elapsed = time.perf_counter() - t_start
    clocks = sampler.stop()
    st = solver.stats()

    # max over ranks of the device and host times
    tot_dev = sum(dev_ms) / 1e3
    tot_wall = sum(wall)
    tot_dev, tot_wall, elapsed = max_over_ranks([tot_dev, tot_wall, elapsed], dist, dev)
    units = ncand * world * args.steps
    value = units / tot_dev
    e2e = units / tot_wall

    # roofline of the advance kernel (average launch over the timed region)
    launches = st["launches"]
    cells_per_launch = st["cell_updates"] / launches   # solves * nx * ny * T (average over launches)
    launch_s = (sum(adv_ms) / len(adv_ms)) / 1e3 / launches
    achieved = BYTES_PER_CELL_UPDATE * cells_per_launch / launch_s / 1e9
    peaks = _peaks()
    tr = _profile_traffic(st["steps_per_launch"], st["cols_per_lane"], st.get("min_blocks_per_sm", 2))
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                "frac": achieved / peaks["hbm_gbs"], "peak_source": peaks["source"],
                "traffic": (tr * cells_per_launch) if tr is not None else None,
                "algorithmic_bytes_per_launch": BYTES_PER_CELL_UPDATE * cells_per_launch,
                "kernel": "fdtd_advance_kernel<float,%d,%d> (min %d blocks/SM)" % (
                    st["steps_per_launch"], st["cols_per_lane"], st.get("min_blocks_per_sm", 2))}
    gcells = st["cell_updates"] * world * args.steps / tot_dev / 1e9

    extra = {}
    if rank == 0 and world == 1 and not args.no_extras:
        # FP64 plain path: one solve per launch, one launch per field update and
        # time step (H, E, DFT), no temporal blocking, no graph -- the denominator
        # of the batching + precision speed-up, timed per candidate (16 solves)
        pspec = spec.copy(precision=T.FP64, plain=1)
        plain_ms = []
        with T.Solver(pspec) as ps:
            ps.set_target(target)
            ps.fitness(cands[0])   # warm-up
            for k in range(3):
                ps.fitness(cands[k])
                plain_ms.append(ps.stats()["total_ms"])
            out64 = ps.forward(cands[:1], traces=False, traces_f64=True, far_field=False, fitness=True)
            pst = ps.stats()
        plain_ms.sort()
        plain_s = plain_ms[len(plain_ms) // 2] / 1e3
        out32 = solver.forward(cands[:1], traces=True, far_field=False, fitness=True)
        tr64 = out64["traces_f64"][0]
        err = float(np.linalg.norm(out32["traces"][0].astype(np.float64) - tr64) / np.linalg.norm(tr64))
        ferr = float(abs(out32["fitness"][0] - out64["fitness"][0]) / abs(out64["fitness"][0]))
        extra["fp64_plain"] = {"evals_per_s": 1.0 / plain_s, "speedup_of_value": value / (1.0 / plain_s),
                               "speedup_of_e2e": e2e / (1.0 / plain_s),
                               "latency_ms": {"p50": plain_ms[len(plain_ms) // 2], "max": plain_ms[-1]},
                               "gcell_updates_per_s": pst["cell_updates"] / (plain_s * 1e9),
                               "kernels_per_eval": int(pst["kernels"]),
                               "what": "FP64, one solve per launch, H/E/DFT kernel per step, no graph; device time "
                                       "per candidate (16 solves), median of 3"}
        extra["error_vs_fp64"] = {"trace_rel_l2": err, "fitness_rel": ferr, "candidates": 1}
        extra["fitness_head"] = [float(v) for v in fit[:4]]
        # reported CPU baseline: oracle FP32 port of the reference CPU solver
        threads = os.cpu_count() or 1
        cb, info = cpu_baseline_sample(spec.as_dict(), cands[0], threads)
        # a bounded sample of the serving workload (continuous batching of
        # requests of mixed grids at Poisson arrivals), so that per-request and
        # per-evaluation latency are part of every default run
        if args.serving_requests > 0:
            extra["serving_sample"] = serving_sample(args.serving_requests, 2, 8, 0.8, args.rate_gcells)
        extra["cpu_baseline"] = {"value": cb, "unit": "evals/s", "cores": threads, "kind": "port",
                                 "sample": "1 candidate = 16 transmitter solves (400x400 x 3000 steps), one per "
                                           "host thread, oracle FP32 port of FDTD_CPU.cxx (%.1f s)" % info["seconds"]}

    lat = sorted(w * 1e3 for w in wall)
    line = {
        "metric": METRIC, "value": value, "unit": "evals/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * tot_dev / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded candidates and target phantom)",
        "config": workload_config(world, ncand),
        "tuning": {"steps_per_launch": st["steps_per_launch"], "cols_per_lane": st["cols_per_lane"],
                   "autotune": tune},
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


def run_large(args) -> None:
    """Large-batch workload: 2048x2048 grid, dx 0.125 mm, 16-cell CPML, 20000
    steps, 32 transmitters per candidate, 16 ellipses in a skin-layer disc, NTFF
    at 16 frequencies over 720 angles.  The full 64-candidate batch holds about
    340 GB of state; this times a bounded subset of candidates (all their
    transmitters, full steps) and compares FP32 with the FP64 GPU path on the
    first transmitters of one candidate."""
    rank, world, _ = _rank_info()
    if rank != 0:
        return
    import torch

    torch.cuda.set_device(0)
    import tomography_gb300 as T
    from tomography_gb300 import workloads as W

    spec = T.breast_spec(4)
    if args.large_steps:
        spec = spec.copy(steps=args.large_steps)
    K = spec.n_ellipses
    ncand = args.large_candidates
    cands = W.candidate_batch(4, ncand, K, disc_radius=spec.disc_radius)
    with T.Solver(spec) as s:
        # the autotuner and the graph build run before the timed time loop (advance_ms)
        sampler = ClockSampler(0)
        sampler.start()
        out = s.forward(cands, traces=False, far_field=True)
        clocks = sampler.stop()
        st = s.stats()
    gcells = st["cell_updates"] / (st["advance_ms"] * 1e6)
    # FP32 vs FP64 GPU on the first transmitters of candidate 0
    ntx = args.large_check_tx
    sub = spec.copy(n_tx=ntx)
    res = {}
    for name, prec in (("fp32", T.FP32), ("fp64", T.FP64)):
        with T.Solver(sub.copy(precision=prec)) as s:
            res[name] = s.forward(cands[:1], traces=True, traces_f64=True, far_field=True)
    t32, t64 = res["fp32"]["traces_f64"][0], res["fp64"]["traces_f64"][0]
    d32, d64 = res["fp32"]["D"][0].astype(np.float64), res["fp64"]["D"][0].astype(np.float64)
    line = {
        "metric": "Gcell-updates/s", "value": gcells, "unit": "Gcell-updates/s", "n_gpus": 1, "steps": 1,
        "warmup": 0, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded candidates)",
        "config": {"workload": "large batch: 2048x2048, dx 0.125 mm, 16-cell CPML, %d steps, 32 tx/candidate, "
                               "16 ellipses, NTFF 16 freqs x 720 angles" % spec.steps,
                   "candidates": ncand, "solves": ncand * spec.n_tx,
                   "sample": "%d of the 64 candidates (the full batch needs about 340 GB of state)" % ncand,
                   "steps_per_launch": st["steps_per_launch"], "cols_per_lane": st["cols_per_lane"],
                   "min_blocks_per_sm": st.get("min_blocks_per_sm")},
        "advance_s": st["advance_ms"] / 1e3, "total_s": st["total_ms"] / 1e3,
        "algorithmic_gbs": BYTES_PER_CELL_UPDATE * gcells, "roofline_frac": BYTES_PER_CELL_UPDATE * gcells /
        _peaks()["hbm_gbs"],
        "error_vs_fp64_gpu": {"trace_rel_l2": float(np.linalg.norm(t32 - t64) / np.linalg.norm(t64)),
                              "far_field_rel_l2": float(np.linalg.norm(d32 - d64) / np.linalg.norm(d64)),
                              "subset": "candidate 0, transmitters 0..%d" % (ntx - 1)},
        "fitness_head": None, "D_checksum": float(np.abs(out["D"]).sum()), "clocks": clocks,
    }
    print(json.dumps(line), flush=True)


SERVING_EDGES = (128, 256, 512, 1024)
SERVING_ANTENNAS = (8, 16, 24, 32)


def serving_sample(nreq: int, bmin: int, bmax: int, utilisation: float, rate_gcells: float) -> dict:
    """Serving workload: a differential-evolution-like client emits candidate
    batches at Poisson arrivals; each request has its own grid edge (128..1024,
    breast at 70% of the domain, 4 x edge steps) and antenna count; every
    request is submitted to one device-resident serving loop (continuous
    batching, admission by an HBM budget) and its latency is measured from its
    scheduled arrival to its fitness on the host.  Returns the measurements."""
    import torch

    import tomography_gb300 as T
    from tomography_gb300 import workloads as W

    rng = W.SplitMix64(W.config_seed(3))
    reqs = []
    for _ in range(nreq):
        edge = SERVING_EDGES[min(3, int(4 * rng.uniform()))]
        ant = SERVING_ANTENNAS[min(3, int(4 * rng.uniform()))]
        nb = bmin + min(bmax - bmin, int((bmax - bmin + 1) * rng.uniform()))
        reqs.append((edge, ant, nb))
    # mean service demand -> Poisson rate for the requested utilisation
    cells = [nb * ant * e * e * 4 * e for e, ant, nb in reqs]
    mean_s = (sum(cells) / nreq) / (rate_gcells * 1e9)
    gap = mean_s / utilisation
    t_arr, t = [], 0.0
    for _ in range(nreq):
        t += -gap * np.log(1.0 - rng.uniform())
        t_arr.append(t)

    classes = sorted({(e, a) for e, a, _ in reqs})
    specs = {c: T.serving_spec(*c) for c in classes}
    K = specs[classes[0]].n_ellipses
    solver = T.Solver(specs[classes[0]])
    for c in classes:   # target phantom traces of every request class
        with T.Solver(specs[c].copy(n_ellipses=3)) as ts:
            tgt = ts.forward(W.target_phantom(3, 3), traces=True, far_field=False)["traces"][0]
        solver.set_target_for(specs[c], tgt)
    # distinct seeded candidates per request
    payload = [np.stack([W.candidate_params(W.config_seed(3) + 7919 * i + 1000 * k, K) for k in range(nb)])
               for i, (_, _, nb) in enumerate(reqs)]

    # warm-up: one small request through the loop
    tk = solver.submit(payload[0][:1], spec=specs[classes[0]])
    while solver.poll(tk, 1) is None:
        solver.serve_step()

    sampler = ClockSampler(0)
    sampler.start()
    lat, inflight, nxt, steps = {}, {}, 0, 0
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    while len(lat) < nreq:
        now = time.perf_counter() - t0
        while nxt < nreq and t_arr[nxt] <= now:
            e, a, nb = reqs[nxt]
            inflight[solver.submit(payload[nxt], spec=specs[(e, a)])] = (nxt, nb)
            nxt += 1
        if inflight:
            solver.serve_step()
            steps += 1
            for tkt in list(inflight):
                i, nb = inflight[tkt]
                if solver.poll(tkt, nb) is not None:
                    lat[i] = time.perf_counter() - t0 - t_arr[i]
                    del inflight[tkt]
        elif nxt < nreq:
            time.sleep(max(0.0, min(0.01, t_arr[nxt] - now)))
    torch.cuda.synchronize()
    span = time.perf_counter() - t0
    clocks = sampler.stop()
    solver.close()
    ms = sorted(1e3 * v for v in lat.values())
    # every evaluation of a request finishes with the request
    per_eval = sorted(1e3 * lat[i] for i, (_, _, nb) in enumerate(reqs) for _ in range(nb))
    evals = sum(nb for _, _, nb in reqs)

    def pct(v, q):
        return v[min(len(v) - 1, int(q * len(v)))]

    return {
        "evals_per_s": evals / span, "requests": nreq, "evaluations": evals, "makespan_s": span,
        "latency_ms_per_request": {"p50": pct(ms, 0.5), "p99": pct(ms, 0.99), "max": ms[-1]},
        "latency_ms_per_evaluation": {"p50": pct(per_eval, 0.5), "p99": pct(per_eval, 0.99)},
        "gcell_updates_per_s": sum(cells) / span / 1e9, "serve_steps": steps, "mean_interarrival_s": gap,
        "utilisation_target": utilisation, "clocks": clocks,
        "workload": "Poisson arrivals, per-request grid edge in %s (4 x edge steps, breast at 70%% of the domain), "
                    "antennas in %s, batch U{%d..%d}" % (list(SERVING_EDGES), list(SERVING_ANTENNAS), bmin, bmax),
    }


def run_serving(args) -> None:
    """The serving workload on its own (see serving_sample)."""
    rank, world, _ = _rank_info()
    if rank != 0:
        return
    import torch

    torch.cuda.set_device(0)
    r = serving_sample(args.requests, args.batch_min, args.batch_max, args.utilisation, args.rate_gcells)
    line = {
        "metric": "serving evals/s, p50/p99 request latency", "value": r["evals_per_s"], "unit": "evals/s",
        "n_gpus": 1, "steps": args.requests, "warmup": 1, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded requests, candidates and target phantoms)",
        "config": {"workload": "serving loop: " + r["workload"], "requests": args.requests,
                   "utilisation_target": args.utilisation, "mean_interarrival_s": r["mean_interarrival_s"],
                   "budget_gb": 150,
                   "sample": "%d requests (batch U{%d..%d}) instead of 10k requests of batch U{8..128}, to bound "
                             "the run" % (args.requests, args.batch_min, args.batch_max)},
        "latency_ms": dict(r["latency_ms_per_request"], per="request (scheduled arrival to fitness on the host)"),
        "latency_ms_per_evaluation": r["latency_ms_per_evaluation"],
        "gcell_updates_per_s": r["gcell_updates_per_s"], "serve_steps": r["serve_steps"],
        "makespan_s": r["makespan_s"], "clocks": r["clocks"],
    }
    print(json.dumps(line), flush=True)


def run_plain(args) -> None:
    """The FP64 plain path on its own: the breast workload's 400x400 grid, one
    candidate (16 transmitter solves), one solve per launch sequence and one
    launch per field update and step (H, E, running DFT), no graph.  One
    untimed forward, then --steps timed forwards; per-step device time is the
    forward's device time over solves x steps."""
    rank, world, _ = _rank_info()
    if rank != 0:
        return
    import torch

    torch.cuda.set_device(0)
    import tomography_gb300 as T
    from tomography_gb300 import workloads as W

    spec = T.breast_spec(CONFIG_INDEX).copy(precision=T.FP64, plain=1)
    if args.plain_steps:
        spec = spec.copy(steps=args.plain_steps)
    cands = W.candidate_batch(CONFIG_INDEX, 1, spec.n_ellipses)
    ms = []
    with T.Solver(spec) as s:
        s.forward(cands, traces=True, far_field=False)
        for _ in range(args.steps):
            s.forward(cands, traces=True, far_field=False)
            ms.append(s.stats()["total_ms"])
        st = s.stats()
    ms.sort()
    med = ms[len(ms) // 2]
    nsolve = spec.n_tx
    line = {
        "metric": "evals/s (FP64 plain path)", "value": 1e3 / med, "unit": "evals/s",
        "n_gpus": 1, "steps": args.steps, "warmup": 1, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded candidate)",
        "config": {"workload": "breast imaging 400x400, %d steps, 1 candidate x %d transmitters, plain FP64 path"
                               % (spec.steps, nsolve)},
        "us_per_step": med * 1e3 / (nsolve * spec.steps), "kernels_per_eval": int(st["kernels"]),
        "gcell_updates_per_s": st["cell_updates"] / (med * 1e6),
    }
    print(json.dumps(line), flush=True)


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--candidates", type=int, default=N_CAND)
    ap.add_argument("--no-extras", action="store_true")
    ap.add_argument("--workload", default="pso", choices=["pso", "serving", "large", "cpu-reference", "plain"])
    ap.add_argument("--plain-steps", type=int, default=0, help="plain: override the 3000 steps")
    ap.add_argument("--cpu-steps", type=int, default=2000, help="cpu-reference: steps timed per copy")
    ap.add_argument("--large-steps", type=int, default=0, help="large: override the 20000 steps")
    ap.add_argument("--large-candidates", type=int, default=2, help="large: candidates timed")
    ap.add_argument("--large-check-tx", type=int, default=2, help="large: transmitters compared with FP64")
    ap.add_argument("--requests", type=int, default=40, help="serving: requests in the sample")
    ap.add_argument("--serving-requests", type=int, default=24,
                    help="default run: requests of the bounded serving sample in the extras (0: none)")
    ap.add_argument("--batch-min", type=int, default=2, help="serving: smallest candidate batch")
    ap.add_argument("--batch-max", type=int, default=16, help="serving: largest candidate batch")
    ap.add_argument("--utilisation", type=float, default=0.8, help="serving: offered load / capacity")
    ap.add_argument("--rate-gcells", type=float, default=120.0,
                    help="serving: capacity (Gcell-updates/s, about the batch path's measured rate) that, "
                         "with --utilisation, sets the arrival rate")
    args = ap.parse_args()
    if args.workload == "cpu-reference":
        run_cpu_reference(args)
    elif args.workload == "serving" and args.impl == "ours":
        run_serving(args)
    elif args.workload == "large" and args.impl == "ours":
        run_large(args)
    elif args.workload == "plain" and args.impl == "ours":
        run_plain(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
