#!/usr/bin/env python
"""FDTD stepping throughput on GB300: one JSON line per run.

Default workload: the 192^3 (7,077,888-cell) sphere under a 10-cell PML with eight DFT
objects (six flux planes, two 32^3 field volumes, 100 frequencies each). One "step" is
one FDTD time step over the whole grid (two fused kernels, plus the monitor kernel on
decimated steps).

* ``value``: Mcell-steps/s with every array resident in HBM, K steps timed with CUDA
  events on the launching stream (the working set, ~1.5 GB, is far above the 129 MB
  L2, so nothing is served from L2 between steps).
* ``e2e``: the same metric through the public API (``FdtdDriver``) from host arrays:
  the freeze with its host-to-device uploads, K steps (with their per-step source words
  uploaded from host), and the device-to-host read of every flux spectrum and DFT
  accumulator, on the wall clock.
* ``roofline``: algorithmic bytes per launch of the dominant kernel over its mean
  CUDA-event duration, against the measured HBM copy bandwidth.
* ``cpu_baseline``: the float32 oracle (the C restatement of the reference's array
  path, OpenMP over every host core) on a bounded sample of the same workload.
* ``error``: relative L2 of the fields and flux against the float64 oracle on bounded
  samples, the timed 192^3 eight-DFT workload's own (600 steps) among them.
* ``configs``: the other configurations (the 80^3 sphere, the 192^3 Lorentz slab)
  device-resident over ``--config-steps`` steps, each with its per-half roofline and clocks.
* ``full_run``: each configuration's whole run at its stated step count (80^3: 2000,
  192^3 eight-DFT: 5000, Lorentz: 10,000) with every DFT sample, contraction and spectrum
  read inside the window, device-resident and end to end through ``FdtdDriver``.
* ``adjoint``: the 96^3 adjoint gradient (forward with checkpoints, backward) and its
  agreement with the float64 finite differences of ``tests/golden/adjoint96_fd.json``.
* ``lossy``: the lossy kernels (D and B conductivity) on two 192^3 workloads, an
  absorber in place of the PML and a conductivity under the PML, each with its per-half
  roofline, and their float64 error on a 40^3 lossy case.
* ``complex``: complex fields on the Bloch-periodic 192^3 case (both parts stepped
  together), its per-half roofline, and the float64 error of a complex 80^3 case.
* ``mirror``: the folded path on the headline case under an even Y and an odd Z mirror
  (192 x 97 x 97 stored cells), its throughput on the stored cells and as the unfolded
  run it stands for, its per-half roofline with the fold kernels, and the float64 error
  of the folded 80^3 case.

``--impl reference`` times the reference path's CPU implementation (the oracle port:
the reference itself is Python and does not travel) on the same workload instead.
"""

from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "Mcell-updates/s"


def parse_args():
    p = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=500)
    p.add_argument("--warmup", type=int, default=20)
    p.add_argument("--impl", choices=("gb300", "reference"), default="gb300")
    p.add_argument("--workload", default="sphere192_8dft")
    p.add_argument("--kernels", default=None,
                   help="family,block_z,block_y,x_chunk for both halves, or eight numbers (H half, "
                        "then E half); families 0/2/4/5 generic, 1/3 TMA tiles; default: the "
                        "autotuner's choice")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-validate", action="store_true")
    p.add_argument("--kernel-steps", type=int, default=40, help="steps timed kernel by kernel")
    p.add_argument("--complex-steps", type=int, default=100,
                   help="steps timed on the Bloch-periodic complex bloch192 workload (0: skip)")
    p.add_argument("--mirror-steps", type=int, default=200,
                   help="steps timed on the folded mirror192 workload (0: skip the mirror section)")
    p.add_argument("--lossy-steps", type=int, default=100,
                   help="steps timed on each lossy 192^3 workload (0: skip the lossy section)")
    p.add_argument("--serving", type=int, default=512,
                   help="requests in the served stream (0: skip the serving measurement)")
    p.add_argument("--serving-slots", type=int, default=48)
    p.add_argument("--serving-groups", type=int, default=4,
                   help="independent batches (own stream and graph each) the slots are spread over")
    p.add_argument("--serving-replay", type=int, default=128, help="steps per captured replay")
    p.add_argument("--serving-budget-gb", type=float, default=16.0)
    p.add_argument("--no-plain", action="store_true", help="skip the one-at-a-time solve")
    p.add_argument("--config-steps", type=int, default=200,
                   help="steps timed on the other configurations (80^3 sphere, 192^3 Lorentz slab); 0 skips")
    p.add_argument("--no-full-run", action="store_true",
                   help="skip the whole runs of the three configurations at their stated step counts")
    p.add_argument("--no-adjoint", action="store_true", help="skip the adjoint section of the default line")
    p.add_argument("--adjoint", action="store_true",
                   help="instead of the step line: the 96^3 adjoint-gradient workload")
    p.add_argument("--dft", action="store_true",
                   help="instead of the step line: the tensor-core DFT contraction on a flux plane")
    p.add_argument("--fd-voxels", type=int, default=4,
                   help="voxels checked by float64 central differences in --adjoint mode")
    return p.parse_args()


def max_over_ranks(value: float, device, world: int) -> float:
    """The largest of every rank's value (the job's time is its slowest replica's)."""
    if world <= 1:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def step_launches(engine, first: int, steps: int) -> int:
    """Kernels of ours that steps first .. first+steps-1 launch: the two halves, and per
    monitor due after a step either its accumulation (step by step) or its sample plus,
    every MGB_DFT_DEPTH samples, a phase table and a contraction per time group (E, H)."""
    from meep_gpu_gb300 import _lib
    # the two halves, each as one launch or as one launch per x range
    count = 2 * steps * max(1, getattr(engine, "split", 0) or 1)
    for index, m in enumerate(engine.monitors):
        due = sum(1 for n in range(first, first + steps) if (n + 1) % m.decimation_factor == 0)
        if engine.dft_samples[index] is None:
            count += due
            continue
        pending = engine.lib.mgb_dft_pending(engine.handle, index)
        groups = len({c[0] for c in m.components})  # "E" and/or "H"
        flushes = (pending + due) // _lib.MGB_DFT_DEPTH
        count += due + flushes * 2 * groups
    return count


def family_name(choice) -> str:
    """(family, block_z, block_y, x_chunk) as words."""
    family, bz, by, xc = choice
    if family == 1:
        return f"tiles 64x8, x chunk {xc}"
    if family == 3:
        return f"warp-specialized tiles 64x8, x chunk {xc}"
    words = f"{'prefetching ' if family in (2, 5) else ''}generic {bz}x{by}, x chunk {xc}"
    return words + (" prefetched into L2" if family in (4, 5) else "")


def measured_peaks():
    path = ROOT / "MEASURED_PEAKS.json"
    if path.exists():
        data = json.loads(path.read_text())
        return float(data["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
            time.sleep(0.25)
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            time.sleep(0.15)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        return False

    def summary(self):
        if not self.lines:
            return None
        sm, sm_max, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [v.strip() for v in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                sm_max = max(sm_max, float(parts[2]))
            except ValueError:
                continue
            for name, flag in zip(names, parts[5:9]):
                if flag.lower() == "active":
                    reasons.add(name)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": sm_max, "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_threads() -> int:
    return os.cpu_count() or 1


def time_oracle(workload: str, steps: int, budget_s: float = 20.0, warmup: int = 1):
    """Float32 oracle Mcell-steps/s on ``steps`` steps (capped to a ~``budget_s`` sample),
    after ``warmup`` untimed steps (also capped to the budget)."""
    from meep_gpu_gb300 import FdtdDriver, workloads
    from oracle.oracle import Oracle, problem_from_driver
    os.environ.setdefault("OMP_NUM_THREADS", str(cpu_threads()))
    driver, _, _ = workloads.build(workload, FdtdDriver)
    oracle = Oracle(problem_from_driver(driver), "f32")
    oracle.run(1)  # warm-up (page-in, thread pool)
    t0 = time.perf_counter()
    oracle.run(1)
    first = max(time.perf_counter() - t0, 1e-6)
    extra = max(0, min(warmup - 2, int(0.25 * budget_s / first)))
    if extra:
        oracle.run(extra)
    t0 = time.perf_counter()
    oracle.run(1)
    per_step = max(time.perf_counter() - t0, 1e-6)
    sample = max(1, min(steps, int(budget_s / per_step)))
    t0 = time.perf_counter()
    oracle.run(sample)
    elapsed = time.perf_counter() - t0
    cells = driver.grid.total_cells
    return cells * sample / elapsed / 1e6, sample, cells


def workload_config(workload: str, cells: int, world: int) -> dict:
    """The ``config`` object both arms print (the same keys and values)."""
    return {"workload": workload, "cells": cells, "parallelism": f"replicas{world}",
            "l2": "inputs larger than L2 (no flush needed)"}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    value, sample, cells = time_oracle(args.workload, max(args.steps, 1), budget_s=60.0, warmup=args.warmup)
    line = {
        "impl": "reference", "metric": METRIC, "value": round(value, 3), "unit": "Mcell-steps/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(cells / (value * 1e6) * 1e3, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": workload_config(args.workload, cells, args.gpus),
        "cpu_baseline": {"value": round(value, 3), "unit": "Mcell-steps/s", "cores": cpu_threads(),
                         "kind": "port",
                         "sample": f"{sample} full-grid steps of {args.workload} on the float32 C oracle "
                                   f"(OpenMP, {cpu_threads()} threads), timed after the warm-up"},
        "e2e": {"value": round(value, 3), "unit": "Mcell-steps/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    if "--adjoint" in sys.argv:
        return bench_adjoint(parse_args())
    if "--dft" in sys.argv:
        return bench_dft(parse_args())
    args = parse_args()
    if args.impl == "reference":
        run_reference(args)
        return
    import torch

    from meep_gpu_gb300 import FdtdDriver, workloads

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    device = torch.device("cuda", local)
    kernels = None
    if args.kernels:
        values = tuple(int(v) for v in args.kernels.split(","))
        # four numbers: one choice for both halves; eight: the H half's, then the E half's
        kernels = values if len(values) == 4 else (values[:4], values[4:])

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    # ---- device-resident throughput ---------------------------------------------------
    driver, flux, dft = workloads.build(args.workload, FdtdDriver, gpu_id=local, kernels=kernels)
    driver.step_many(args.warmup)  # freezes the configuration and warms the kernels
    engine = driver.engine
    choice = list(engine.choice) if engine.choice is not None else None
    split, wave = getattr(engine, "split", 0), getattr(engine, "wave", None)
    cells = driver.grid.total_cells
    first = driver.step_count
    engine.ensure_source_words(first, args.steps)
    stream = torch.cuda.current_stream(device)
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launches = step_launches(engine, first, args.steps)
    torch.cuda.synchronize(device)
    barrier()
    with ClockSampler(local) as clocks:
        start.record(stream)
        engine.step(first, args.steps)
        end.record(stream)
        torch.cuda.synchronize(device)
    driver.step_count += args.steps
    ms = max_over_ranks(start.elapsed_time(end), device, world)
    value = cells * args.steps * world / (ms / 1e3) / 1e6
    if engine.nonfinite():
        raise RuntimeError("the benchmark run wrote a non-finite field")

    # ---- kernel-by-kernel timing (roofline) ---------------------------------------------
    kernel_steps = max(1, args.kernel_steps)
    n0 = driver.step_count
    engine.ensure_source_words(n0, kernel_steps)
    events = [[torch.cuda.Event(enable_timing=True) for _ in range(4)] for _ in range(kernel_steps)]
    torch.cuda.synchronize(device)
    for t in range(kernel_steps):
        ev = events[t]
        ev[0].record(stream)
        engine.launch(n0 + t, 0, stream)
        ev[1].record(stream)
        engine.launch(n0 + t, 1, stream)
        ev[2].record(stream)
        engine.launch(n0 + t, 2, stream)
        ev[3].record(stream)
    torch.cuda.synchronize(device)
    driver.step_count += kernel_steps
    h_ms = float(np.mean([e[0].elapsed_time(e[1]) for e in events]))
    e_ms = float(np.mean([e[1].elapsed_time(e[2]) for e in events]))
    bytes_per = engine.algorithmic_bytes()
    peak, peak_kind = measured_peaks()
    timed = {"h_half": {"ms": h_ms, "bytes": bytes_per["h_half"]},
             "e_half": {"ms": e_ms, "bytes": bytes_per["e_half"]}}
    for info in timed.values():
        info["gbs"] = info["bytes"] / (info["ms"] / 1e3) / 1e9
    dominant = max(timed, key=lambda k: timed[k]["ms"])
    traffic = None
    summary = ROOT / "profiles" / f"{dominant}_{args.workload}.txt"
    if summary.exists():
        for line in summary.read_text().splitlines():
            if line.startswith("traffic_bytes_per_launch:"):
                traffic = int(float(line.split(":", 1)[1]))
    step_bytes = bytes_per["h_half"] + bytes_per["e_half"]
    roofline = {"bound": "hbm", "kernel": dominant,
                "achieved": round(timed[dominant]["gbs"], 1), "peak": peak, "unit": "GB/s",
                "frac": round(timed[dominant]["gbs"] / peak, 4), "traffic": traffic,
                "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else "fallback",
                "algorithmic_bytes_per_launch": bytes_per[dominant],
                "per_kernel": {k: {"ms": round(v["ms"], 4), "GB/s": round(v["gbs"], 1),
                                   "frac": round(v["gbs"] / peak, 4)} for k, v in timed.items()},
                "step_bytes_per_cell": round(step_bytes / cells, 2),
                "step_frac": round(step_bytes / ((ms / args.steps) / 1e3) / 1e9 / peak, 4),
                "bytes_counted": "words the step moves; the f_w words of H and E, which the "
                                 "reference also moves, are formed in registers and not counted"}
    driver.close()
    del driver, engine
    torch.cuda.empty_cache()

    # ---- end to end through the public API ---------------------------------------------
    e2e = None
    if not args.no_e2e:
        torch.cuda.synchronize(device)
        barrier()
        t0 = time.perf_counter()
        d2, f2, v2 = workloads.build(args.workload, FdtdDriver, gpu_id=local, kernels=kernels)
        d2.run(num_steps=args.steps, progress_interval=max(args.steps, 1), check_finite=False)
        results = [m.get_flux_spectrum() for m in f2]
        arrays = [m.raw(c) for m in v2 for c in m.components]
        torch.cuda.synchronize(device)
        wall = time.perf_counter() - t0
        eng = d2.engine
        h2d = sum(int(t.numel() * t.element_size()) for t in eng.inv_eps[:1])
        h2d += sum(int(t.numel() * t.element_size()) for t in eng.coefficients.values())
        h2d += 8 * eng.desc.nsrc * args.steps
        d2h = sum(r.nbytes for r in results) + sum(a.nbytes for a in arrays)
        e2e = {"value": round(cells * args.steps * world / wall / 1e6, 3), "unit": "Mcell-steps/s",
               "h2d_bytes_per_step": int(h2d / args.steps), "d2h_bytes_per_step": int(d2h / args.steps),
               "wall_s": round(wall, 3),
               "what": "FdtdDriver from host arrays: freeze + uploads, K steps, read every flux "
                       "spectrum and DFT accumulator"}
        d2.close()
        del d2, eng
        torch.cuda.empty_cache()

    if rank != 0:
        return
    # ---- CPU baseline and float64 error (rank 0 only) -----------------------------------
    cpu = None
    if not args.no_cpu_baseline:
        cpu_value, sample, _ = time_oracle(args.workload, args.steps, budget_s=20.0)
        cpu = {"value": round(cpu_value, 3), "unit": "Mcell-steps/s", "cores": cpu_threads(),
               "kind": "port",
               "sample": f"{sample} full-grid steps of {args.workload} on the float32 C oracle "
                         f"(OpenMP, {cpu_threads()} threads)"}
    error = None
    if not args.no_validate:
        error = validate(device)
    configs = None
    if args.config_steps > 0:
        configs = {name: measure_workload(device, name, args.config_steps) for name in ("sphere80", "lorentz192")}
    full_run = None
    if not args.no_full_run:
        full_run = {name: bench_full_run(device, name) for name in ("sphere80", "sphere192_8dft", "lorentz192")}
    adjoint = None
    if not args.no_adjoint:
        adjoint = adjoint_section(args)
    served = None
    if args.serving > 0:
        served = bench_serving(device, args)
    lossy = None
    mirror = None
    complex_ = None
    if args.lossy_steps > 0:
        lossy = bench_lossy(device, args)
    if args.mirror_steps > 0:
        mirror = bench_mirror(device, args)
    if args.complex_steps > 0:
        complex_ = bench_complex(device, args)
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": "Mcell-steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms / args.steps, 5),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": workload_config(args.workload, cells, world),
        "kernels": {"h_half": family_name(choice[0]) if choice else None,
                    "e_half": family_name(choice[1]) if choice else None,
                    "choice": choice, "x_range_split": split, "wave": wave,
                    "chosen_by": "argument" if kernels else "autotuner"},
        "monitors": {"flux_planes": len(flux), "dft_volumes": len(dft),
                     "decimation": [m.decimation_factor for m in list(flux) + list(dft)][:1]},
        "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": launches,
        "clocks": clocks.summary(), "error": error, "configs": configs, "full_run": full_run,
        "adjoint": adjoint, "serving": served, "lossy": lossy, "mirror": mirror, "complex": complex_,
    }
    print(json.dumps(line), flush=True)


def bench_serving(device, args):
    """The mixed-size request stream: continuous batching against one-at-a-time solves.

    Both arms see the same seeded stream with wall-clock Poisson arrivals, build every
    request from host arrays and end with its flux spectrum on the host. Before timing,
    one short request per side runs through both arms (kernel choices, graph capture).
    """
    import torch

    from meep_gpu_gb300 import serving
    requests = serving.make_stream(args.serving, rate=40.0, seed=0)
    warm = [serving.Request(-1 - i, s, 4.0, 0.3 * s, 70, 0.0) for i, s in enumerate(serving.SIDES)]
    server = serving.MultiBatchServer(device, groups=args.serving_groups, max_slots=args.serving_slots,
                                      steps_per_replay=args.serving_replay,
                                      budget_bytes=int(args.serving_budget_gb * 1e9))
    shape = server.autotune()
    serving.serve(server, warm, realtime=False)
    torch.cuda.synchronize(device)
    with ClockSampler(device.index or 0) as clocks:
        report = serving.serve(server, requests, realtime=True)
    server.close()
    cellsteps = sum(r.side ** 3 * r.steps for r in requests)
    out = {
        "requests": len(requests), "arrivals": "Poisson 40/s, seed 0",
        "sides": list(serving.SIDES), "steps": "U[1000,4000]", "pml_cells": serving.PML_CELLS,
        "nfreq": serving.NFREQ, "slots": args.serving_slots, "groups": args.serving_groups,
        "steps_per_replay": args.serving_replay,
        "budget_gb": args.serving_budget_gb, "shape": list(shape), "graph": True,
        "sims_per_s": round(report.sims_per_second, 3),
        "p50_s": round(report.latency_percentile(50), 4),
        "p99_s": round(report.latency_percentile(99), 4),
        "wall_s": round(report.wall_seconds, 3), "replays": report.replays,
        "mcell_steps_per_s": round(cellsteps / report.wall_seconds / 1e6, 1),
        "clocks": clocks.summary(),
    }
    if not args.no_plain:
        serving.solve_plain(warm, realtime=False)
        torch.cuda.synchronize(device)
        plain = serving.solve_plain(requests, realtime=True)
        mine = report.spectra()
        worst = 0.0
        for r in plain.results:
            ref = r.spectrum
            worst = max(worst, float(np.max(np.abs(mine[r.index] - ref)) / max(np.max(np.abs(ref)), 1e-300)))
        out["plain"] = {"sims_per_s": round(plain.sims_per_second, 3),
                        "p50_s": round(plain.latency_percentile(50), 4),
                        "p99_s": round(plain.latency_percentile(99), 4),
                        "wall_s": round(plain.wall_seconds, 3),
                        "what": "FdtdDriver per request, autotuned kernels, step_many + flux read"}
        out["served_vs_plain_max_rel_diff"] = worst
    return out


def bench_adjoint(args):
    """``--adjoint``: the adjoint section alone, as one JSON line."""
    print(json.dumps(adjoint_section(args)), flush=True)


def adjoint_section(args) -> dict:
    """96^3 adjoint gradient: forward with checkpoints, backward, float64 finite differences.

    The objective, the timing of forward and backward (CUDA events around each), and the
    agreement with central differences (h = 1e-3) of the float64 oracle on seeded voxels
    and along one seeded direction over the box (read from the committed fixture when
    present, else computed with ``--fd-voxels`` voxels).
    """
    import torch

    from meep_gpu_gb300 import workloads
    from meep_gpu_gb300.adjoint import FluxAdjoint
    from oracle.oracle import Oracle, problem_from_driver

    device = torch.device("cuda", 0)
    driver, flux, box, eps_box = workloads.adjoint96()
    steps = workloads.ADJOINT96_STEPS
    problem = FluxAdjoint(driver, flux, box, steps, checkpoint_every=200)
    eps = torch.tensor(eps_box, dtype=torch.float64, requires_grad=True)
    problem.forward(torch.from_numpy(eps_box))  # warm-up (kernel choice, plan)
    problem.backward()
    torch.cuda.synchronize(device)
    marks = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    marks[0].record()
    value = problem.objective(eps)
    marks[1].record()
    value.backward()
    marks[2].record()
    torch.cuda.synchronize(device)
    grad = eps.grad.numpy()
    fwd_ms, bwd_ms = marks[0].elapsed_time(marks[1]), marks[1].elapsed_time(marks[2])
    cells = driver.grid.total_cells

    def oracle_j(values):
        d, _, _, _ = workloads.adjoint96(eps_box=values)
        prob = problem_from_driver(d)
        full = np.ones(d.grid.shape)
        (i0, i1), (j0, j1), (k0, k1) = box
        full[i0:i1, j0:j1, k0:k1] = values
        prob.inv_eps64 = [1.0 / full] * 3
        o = Oracle(prob, "f64")
        o.run(steps)
        return float(np.sum(o.flux_spectrum(0)))

    h = 1e-3
    fixture = ROOT / "tests" / "golden" / "adjoint96_fd.json"
    if fixture.exists():
        # float64 central differences recorded by tests/golden/make_adjoint_fd.py, whose
        # voxels and direction come from the same seeded generator as below
        record = json.loads(fixture.read_text())
        count = len(record["voxels"])
    else:
        record, count = None, args.fd_voxels
    rng = np.random.default_rng(0)
    picks = [tuple(int(rng.integers(0, n)) for n in eps_box.shape) for _ in range(count)]
    direction = rng.standard_normal(eps_box.shape)
    direction /= np.linalg.norm(direction)
    if record is not None:
        assert [tuple(v["voxel"]) for v in record["voxels"]] == picks, "fixture voxels differ from the seeds"
        j64 = record["objective"]
        fd = [v["fd"] for v in record["voxels"]]
        fd_dir = record["directional_fd"]
        fd_source = "tests/golden/adjoint96_fd.json (float64 oracle)"
    else:
        def bumped(v, sign):
            values = eps_box.copy()
            values[v] += sign * h
            return values

        j64 = oracle_j(eps_box)
        fd = [(oracle_j(bumped(v, 1)) - oracle_j(bumped(v, -1))) / (2 * h) for v in picks]
        fd_dir = (oracle_j(eps_box + h * direction) - oracle_j(eps_box - h * direction)) / (2 * h)
        fd_source = "float64 oracle, this run"
    ad = [float(grad[v]) for v in picks]
    ad_dir = float(np.sum(grad * direction))
    reverse = adjoint_reverse_roofline(problem, steps)
    line = {
        "metric": "adjoint gradient (96^3, 4000 steps, checkpoints every 200)",
        "objective": float(value.item()), "objective_f64": j64,
        "objective_rel_err": abs(float(value.item()) - j64) / abs(j64),
        "forward_ms": round(fwd_ms, 2), "backward_ms": round(bwd_ms, 2),
        "gradient_ms": round(fwd_ms + bwd_ms, 2),
        "mcell_steps_per_s_forward": round(cells * steps / (fwd_ms / 1e3) / 1e6, 1),
        "fd_voxels": [{"voxel": list(v), "adjoint": a, "fd_f64": f} for v, a, f in zip(picks, ad, fd)],
        "fd_rel_l2": float(np.linalg.norm(np.array(ad) - np.array(fd)) / np.linalg.norm(fd)) if fd else None,
        "directional": {"adjoint": ad_dir, "fd_f64": fd_dir, "rel_err": abs(ad_dir - fd_dir) / abs(fd_dir)},
        "h": h, "fd_source": fd_source, "box": [list(b) for b in box],
        "reverse_step": reverse,
        "data": "synthetic (seeded eps ~ U[1,12])",
        "reference_adjoint": "unavailable: the reference has no adjoint gradient",
    }
    problem.close()
    return line


def adjoint_reverse_roofline(problem, steps: int, reps: int = 60) -> dict:
    """The reverse step alone (``mgb_adjoint_step``: the transposed E half, then the
    transposed H half), timed with CUDA events over ``reps`` reversals of the last step
    after the gradient has been read (the words it leaves are not used), against its
    algorithmic bytes: per cell, the transposed E half reads the adjoint E, D and mu_B (3
    volumes each) and each distinct inverse-epsilon volume and writes E, D and mu_D (3
    each); the transposed H half reads H and mu_D and writes H and mu_B (3 each); on the
    PML slabs each auxiliary the forward half touches is read and written once
    (``fu``/``f_w`` of D and E; ``fu`` of B, the slab B and ``f_w`` of H); over the
    gradient box the saved D (3 words) is read and the gradient read and written."""
    import ctypes

    import torch

    engine = problem.engine
    lib = engine.lib
    stream = problem.stream
    word = 4
    cells = engine.grid.total_cells
    aux = lambda name: sum(engine.aux_cells[f"{name}{a}"] for a in "xyz") if engine.pml is not None else 0  # noqa: E731
    distinct_inv = len({t.data_ptr() for t in engine.inv_eps})
    box_cells = int(np.prod([b1 - b0 for b0, b1 in problem.box]))
    e_bytes = word * ((18 + distinct_inv) * cells + 2 * aux("fuD") + 2 * aux("fwE") + 5 * box_cells)
    h_bytes = word * (12 * cells + 2 * aux("fuB") + 2 * aux("B") + 2 * aux("fwH"))
    args = ctypes.byref(problem.adj)
    handle = stream.cuda_stream
    for _ in range(3):
        _lib_check(lib, lib.mgb_adjoint_step(problem.adj_handle, args, steps - 1, handle))
    marks = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    torch.cuda.synchronize()
    marks[0].record(stream)
    for _ in range(reps):
        _lib_check(lib, lib.mgb_adjoint_step(problem.adj_handle, args, steps - 1, handle))
    marks[1].record(stream)
    torch.cuda.synchronize()
    ms = marks[0].elapsed_time(marks[1]) / reps
    peak, source = measured_peaks()
    gbs = (e_bytes + h_bytes) / (ms / 1e3) / 1e9
    return {"ms": round(ms, 4), "algorithmic_bytes": e_bytes + h_bytes,
            "bytes_e": e_bytes, "bytes_h": h_bytes, "gbs": round(gbs, 1),
            "hbm_frac": round(gbs / peak, 3), "peak_gbs": peak, "peak_source": source,
            "note": f"{reps} reversals of the last step, CUDA events; two launches each"}


def _lib_check(lib, rc):
    from meep_gpu_gb300 import _lib
    _lib.check(lib, rc)


def bench_dft(args):
    """The tensor-core DFT contraction at the size of one 192^3 flux plane.

    One launch adds K = 32 buffered samples of one component (2 x 170 x 170 region cells,
    the plane one cell inside a 10-cell PML at 192^3) into 100 frequencies of
    accumulators. Algorithmic work per launch: 3 TF32 products (3xTF32) of a
    [2 nfreq x K] x [K x N] contraction, 6 * 2 * nfreq * K * N flops; algorithmic bytes:
    the samples read once (K * N words) and the accumulators read and written once
    (2 * 2 * nfreq * N words). Timed with CUDA events over 24 launches after 6 warm-up,
    cycling six sets of buffers (more than L2 holds).
    """
    import torch

    from meep_gpu_gb300 import _lib
    lib = _lib.load()
    nfreq, depth = 100, _lib.MGB_DFT_DEPTH
    ncols = 2 * 170 * 170
    rng = np.random.default_rng(0)
    # six planes' worth of samples and accumulators (~320 MB), cycled, so every launch
    # meets them in HBM rather than in the 129 MB L2
    sets = 6
    samples = [torch.from_numpy(rng.standard_normal((depth, ncols)).astype(np.float32)).cuda() for _ in range(sets)]
    omega = torch.from_numpy(np.linspace(0.6, 1.3, nfreq)).cuda()
    accs = [torch.zeros((2 * nfreq, ncols), dtype=torch.float32, device="cuda") for _ in range(sets)]
    scratch = torch.empty(lib.mgb_dft_scratch_bytes(nfreq) // 4, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()
    turn = [0]

    def launch():
        q = turn[0] % sets
        turn[0] += 1
        _lib.check(lib, lib.mgb_dft_contract(samples[q].data_ptr(), ncols, ncols, depth, omega.data_ptr(), nfreq,
                                             120, 120, 0.5 / 24, 0, 0.1, accs[q].data_ptr(), scratch.data_ptr(),
                                             scratch.numel() * 4, stream.cuda_stream))

    for _ in range(sets):
        launch()
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = 24
    start.record(stream)
    for _ in range(reps):
        launch()
    end.record(stream)
    end.synchronize()
    ms = start.elapsed_time(end) / reps
    flops = 6.0 * 2 * nfreq * depth * ncols
    nbytes = 4.0 * (depth * ncols + 2 * 2 * nfreq * ncols)
    peak, kind = measured_peaks()
    line = {"metric": "tensor-core DFT contraction (3xTF32)", "nfreq": nfreq, "depth": depth, "columns": ncols,
            "ms_per_launch": round(ms, 4), "tflops": round(flops / (ms / 1e3) / 1e12, 2),
            "gbs": round(nbytes / (ms / 1e3) / 1e9, 1), "hbm_frac": round(nbytes / (ms / 1e3) / 1e9 / peak, 3),
            "hbm_peak": peak, "peak_source": kind,
            "note": "phase table kernel included in each launch; six buffer sets cycled (larger than L2)"}
    print(json.dumps(line), flush=True)


def measure_workload(device, name: str, steps: int, kernel_steps: int = 20) -> dict:
    """One workload device-resident: ``steps`` steps timed with CUDA events on the
    launching stream after 3 warm-up steps, then each half timed launch by launch over
    ``kernel_steps`` steps; per-half and whole-step roofline against the measured HBM
    peak, with the clocks sampled during the timed steps."""
    import torch

    from meep_gpu_gb300 import FdtdDriver, workloads

    peak, _ = measured_peaks()
    stream = torch.cuda.current_stream(device)
    driver, _, _ = workloads.build(name, FdtdDriver)
    driver.step_many(3)
    engine = driver.engine
    first = driver.step_count
    engine.ensure_source_words(first, steps + kernel_steps)
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize(device)
    with ClockSampler(device.index or 0) as clocks:
        start.record(stream)
        engine.step(first, steps)
        end.record(stream)
        torch.cuda.synchronize(device)
    ms = start.elapsed_time(end) / steps
    n0 = first + steps
    events = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(kernel_steps)]
    for t, ev in enumerate(events):
        ev[0].record(stream)
        engine.launch(n0 + t, 0, stream)
        ev[1].record(stream)
        engine.launch(n0 + t, 1, stream)
        ev[2].record(stream)
    torch.cuda.synchronize(device)
    nbytes = engine.algorithmic_bytes()
    halves = {}
    for part, key in enumerate(("h_half", "e_half")):
        half_ms = float(np.mean([ev[part].elapsed_time(ev[part + 1]) for ev in events]))
        gbs = nbytes[key] / (half_ms / 1e3) / 1e9
        halves[key] = {"ms": round(half_ms, 4), "GB/s": round(gbs, 1), "frac": round(gbs / peak, 4)}
    cells = driver.grid.total_cells
    step_bytes = nbytes["h_half"] + nbytes["e_half"]
    out = {"value": round(cells / (ms / 1e3) / 1e6, 3), "unit": "Mcell-steps/s", "cells": cells,
           "ms_per_step": round(ms, 5), "steps": steps, "step_bytes_per_cell": round(step_bytes / cells, 2),
           "step_frac": round(step_bytes / (ms / 1e3) / 1e9 / peak, 4), "per_kernel": halves,
           "kernels": [list(c) for c in engine.choice] if engine.choice is not None else None,
           "clocks": clocks.summary()}
    if engine.nonfinite():
        raise RuntimeError(f"the {name} run wrote a non-finite field")
    driver.close()
    del driver, engine
    torch.cuda.empty_cache()
    return out


def bench_full_run(device, name: str) -> dict:
    """A configuration's whole run at its stated step count, every monitor included.

    ``device``: steps 0 .. N-1 of a fresh driver (kernels chosen at the freeze on a
    scratch copy) timed with CUDA events, with every DFT sample, contraction and the
    final read of every spectrum inside the window. ``e2e``: the same run through the
    public API from host arrays (``FdtdDriver``: configure, ``run(num_steps=N)`` with its
    default checks, read every flux spectrum and DFT array), on the wall clock.
    """
    import torch

    from meep_gpu_gb300 import FdtdDriver, workloads

    total = workloads.STEPS[name]
    stream = torch.cuda.current_stream(device)
    driver, flux, dft = workloads.build(name, FdtdDriver)
    engine = driver.freeze()
    engine.ensure_source_words(0, total)
    launches = step_launches(engine, 0, total)
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize(device)
    with ClockSampler(device.index or 0) as clocks:
        start.record(stream)
        engine.step(0, total)
        driver.step_count = total
        spectra = [engine.queue_flux_spectrum(m) for m in flux]
        arrays = [engine.device_accumulator(m, q) for m in dft for q in range(len(m.components))]
        end.record(stream)
        torch.cuda.synchronize(device)
    ms = start.elapsed_time(end)
    cells = driver.grid.total_cells
    finite = all(bool(torch.isfinite(a).all()) for a in arrays)
    driver.close()
    del driver, engine, spectra, arrays
    torch.cuda.empty_cache()
    torch.cuda.synchronize(device)
    t0 = time.perf_counter()
    d2, f2, v2 = workloads.build(name, FdtdDriver)
    d2.run(num_steps=total)
    results = [m.get_flux_spectrum() for m in f2]
    host = [m.raw(c) for m in v2 for c in m.components]
    wall = time.perf_counter() - t0
    d2h = sum(r.nbytes for r in results) + sum(a.nbytes for a in host)
    d2.close()
    del d2
    torch.cuda.empty_cache()
    return {"steps": total, "cells": cells, "ms": round(ms, 2),
            "value": round(cells * total / (ms / 1e3) / 1e6, 1), "unit": "Mcell-steps/s",
            "gpu_launches": launches, "monitors": {"flux_planes": len(flux), "dft_volumes": len(dft)},
            "finite": finite, "clocks": clocks.summary(),
            "e2e": {"value": round(cells * total / wall / 1e6, 1), "unit": "Mcell-steps/s", "wall_s": round(wall, 3),
                    "d2h_bytes": d2h,
                    "what": "FdtdDriver from host arrays: configure, run(num_steps) with its default checks, "
                            "read every spectrum and DFT array"}}


def bench_lossy(device, args):
    """The lossy kernels on the 192^3 absorber and lossy-PML workloads: device-resident
    throughput over K steps, each half's roofline, and the float64 error of the 40^3
    lossy case."""
    import torch

    from meep_gpu_gb300 import FdtdDriver, workloads
    from oracle.oracle import Oracle, problem_from_driver

    out = {name: measure_workload(device, name, args.lossy_steps) for name in ("absorber192", "lossy_pml192")}
    steps = workloads.STEPS["lossy40"]
    gpu, flux, _ = workloads.build("lossy40", FdtdDriver)
    gpu.run(num_steps=steps, progress_interval=steps)
    ref, _, _ = workloads.build("lossy40", FdtdDriver)
    o64 = Oracle(problem_from_driver(ref), "f64")
    o64.run(steps)
    num = den = 0.0
    for c in ("Ex", "Ey", "Ez", "Hx", "Hy", "Hz"):
        a = gpu.get_field(c, cell_centered=False).astype(np.float64)
        b = o64.field(c)
        num += float(np.sum((a - b) ** 2))
        den += float(np.sum(b ** 2))
    got = flux[0].get_flux_spectrum()
    expected = o64.flux_spectrum(0)
    out["error"] = {"lossy40_300_steps": {
        "fields_rel_l2_vs_f64": float(math.sqrt(num / den)),
        "flux_rel_vs_f64": float(np.max(np.abs(got - expected)) / np.max(np.abs(expected)))}}
    gpu.close()
    return out


def bench_complex(device, args):
    """Complex fields: bloch192 (the 192^3 sphere on a lattice periodic in x and y with a
    Bloch vector, the two parts stepped together) device-resident over K steps, each half
    of both parts timed with events; the float64 error of the complex (k = 0) 80^3 case
    (its two parts against two float64 oracle runs) and of the Bloch 48^3 case (against
    the float64 oracle's two parts stepped together)."""
    import torch

    from meep_gpu_gb300 import FdtdDriver, workloads
    from oracle.oracle import BlochPair, Oracle, complex_flux_spectrum, problem_from_driver

    peak, _ = measured_peaks()
    stream = torch.cuda.current_stream(device)
    driver, _, _ = workloads.build("bloch192", FdtdDriver)
    driver.step_many(3)
    engine = driver.engine
    first, steps = driver.step_count, args.complex_steps
    engine.ensure_source_words(first, steps + 20)
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize(device)
    with ClockSampler(device.index or 0) as clocks:
        start.record(stream)
        engine.step(first, steps)
        end.record(stream)
        torch.cuda.synchronize(device)
    ms = start.elapsed_time(end) / steps
    n0 = first + steps
    events = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(20)]
    for t, ev in enumerate(events):
        ev[0].record(stream)
        engine.launch(n0 + t, 0, stream)
        ev[1].record(stream)
        engine.launch(n0 + t, 1, stream)
        ev[2].record(stream)
    torch.cuda.synchronize(device)
    # both parts move the real plan's bytes (the phased reads of the other part touch one
    # plane per phased axis)
    nbytes = {k: 2 * v for k, v in engine.re.algorithmic_bytes().items()}
    halves = {}
    for part, key in enumerate(("h_half", "e_half")):
        half_ms = float(np.mean([ev[part].elapsed_time(ev[part + 1]) for ev in events]))
        gbs = nbytes[key] / (half_ms / 1e3) / 1e9
        halves[key] = {"ms": round(half_ms, 4), "GB/s": round(gbs, 1), "frac": round(gbs / peak, 4)}
    cells = driver.grid.total_cells
    step_bytes = nbytes["h_half"] + nbytes["e_half"]
    out = {"bloch192": {
        "value": round(cells / (ms / 1e3) / 1e6, 3), "unit": "Mcell-steps/s (complex cells)",
        "ms_per_step": round(ms, 5), "steps": steps, "k_point": list(driver.grid.k_point),
        "step_frac": round(step_bytes / (ms / 1e3) / 1e9 / peak, 4), "per_kernel": halves,
        "kernels": [list(c) for c in engine.choice], "clocks": clocks.summary(),
        "note": "two float32 parts per complex word, stepped together (mgb_step_pair)"}}
    if engine.re.nonfinite() or engine.im.nonfinite():
        raise RuntimeError("the bloch192 run wrote a non-finite field")
    driver.close()
    del driver, engine
    torch.cuda.empty_cache()
    steps = workloads.STEPS["complex80"]
    gpu, flux, _ = workloads.build("complex80", FdtdDriver)
    gpu.run(num_steps=steps, progress_interval=steps)
    ref, _, _ = workloads.build("complex80", FdtdDriver)
    problem = problem_from_driver(ref)
    parts = [Oracle(problem, "f64", part) for part in ("real", "imag")]
    for oracle in parts:
        oracle.run(steps)
    num = den = 0.0
    for c in ("Ex", "Ey", "Ez", "Hx", "Hy", "Hz"):
        a = gpu.get_field(c, cell_centered=False).astype(np.complex128)
        b = parts[0].field(c) + 1j * parts[1].field(c)
        num += float(np.sum(np.abs(a - b) ** 2))
        den += float(np.sum(np.abs(b) ** 2))
    got = flux[0].get_flux_spectrum()
    expected = complex_flux_spectrum(parts[0], parts[1], 0)
    out["error"] = {"complex80_600_steps": {
        "fields_rel_l2_vs_f64": float(math.sqrt(num / den)),
        "flux_rel_vs_f64": float(np.max(np.abs(got - expected)) / np.max(np.abs(expected)))}}
    gpu.close()
    # a Bloch run against the float64 oracle's two parts stepped together
    steps = workloads.STEPS["bloch48"]
    gpu, flux, _ = workloads.build("bloch48", FdtdDriver)
    gpu.run(num_steps=steps, progress_interval=steps)
    ref, _, _ = workloads.build("bloch48", FdtdDriver)
    pair = BlochPair(problem_from_driver(ref), "f64")
    pair.run(steps)
    num = den = 0.0
    for c in ("Ex", "Ey", "Ez", "Hx", "Hy", "Hz"):
        a = gpu.get_field(c, cell_centered=False).astype(np.complex128)
        b = pair.field(c)
        num += float(np.sum(np.abs(a - b) ** 2))
        den += float(np.sum(np.abs(b) ** 2))
    got = flux[0].get_flux_spectrum()
    expected = complex_flux_spectrum(pair.re, pair.im, 0)
    out["error"]["bloch48_600_steps"] = {
        "fields_rel_l2_vs_f64": float(math.sqrt(num / den)),
        "flux_rel_vs_f64": float(np.max(np.abs(got - expected)) / np.max(np.abs(expected)))}
    gpu.close()
    return out


def bench_mirror(device, args):
    """The folded path on mirror192 (the headline case under an even Y and an odd Z
    mirror): device-resident throughput over K steps on the stored cells and as the
    unfolded run it stands for, each half's roofline (the fold kernels included in their
    half), and the float64 error of the folded 80^3 case."""
    import torch

    from meep_gpu_gb300 import FdtdDriver, workloads
    from oracle.oracle import Oracle, problem_from_driver

    peak, _ = measured_peaks()
    stream = torch.cuda.current_stream(device)
    driver, _, _ = workloads.build("mirror192", FdtdDriver)
    driver.step_many(3)
    engine = driver.engine
    first, steps = driver.step_count, args.mirror_steps
    engine.ensure_source_words(first, steps + 20)
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize(device)
    with ClockSampler(device.index or 0) as clocks:
        start.record(stream)
        engine.step(first, steps)
        end.record(stream)
        torch.cuda.synchronize(device)
    ms = start.elapsed_time(end) / steps
    n0 = first + steps
    events = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(20)]
    for t, ev in enumerate(events):
        ev[0].record(stream)
        engine.launch(n0 + t, 0, stream)
        ev[1].record(stream)
        engine.launch(n0 + t, 1, stream)
        ev[2].record(stream)
    torch.cuda.synchronize(device)
    nbytes = engine.algorithmic_bytes()
    halves = {}
    for part, key in enumerate(("h_half", "e_half")):
        half_ms = float(np.mean([ev[part].elapsed_time(ev[part + 1]) for ev in events]))
        gbs = nbytes[key] / (half_ms / 1e3) / 1e9
        halves[key] = {"ms": round(half_ms, 4), "GB/s": round(gbs, 1), "frac": round(gbs / peak, 4)}
    cells = driver.grid.total_cells
    full = int(np.prod(driver.grid.shape_full))
    step_bytes = nbytes["h_half"] + nbytes["e_half"]
    out = {"mirror192": {
        "value": round(cells / (ms / 1e3) / 1e6, 3), "unit": "Mcell-steps/s (stored cells)",
        "unfolded_equivalent": round(full / (ms / 1e3) / 1e6, 3),
        "stored_cells": cells, "unfolded_cells": full, "ms_per_step": round(ms, 5), "steps": steps,
        "step_frac": round(step_bytes / (ms / 1e3) / 1e9 / peak, 4), "per_kernel": halves,
        "ghosts": [int(engine.desc.fold.count[0]), int(engine.desc.fold.count[1])],
        "kernels": [list(c) for c in engine.choice], "x_range_split": engine.split, "clocks": clocks.summary(),
        "note": "each half's time includes its fold kernel (ghost words and their E/H); the per-half "
                "times are single launches, the step takes the x-range split"}}
    if engine.nonfinite():
        raise RuntimeError("the mirror192 run wrote a non-finite field")
    driver.close()
    del driver, engine
    torch.cuda.empty_cache()
    steps = workloads.STEPS["mirror80"]
    gpu, flux, _ = workloads.build("mirror80", FdtdDriver)
    gpu.run(num_steps=steps, progress_interval=steps)
    ref, _, _ = workloads.build("mirror80", FdtdDriver)
    o64 = Oracle(problem_from_driver(ref), "f64")
    o64.run(steps)
    num = den = 0.0
    for c in ("Ex", "Ey", "Ez", "Hx", "Hy", "Hz"):
        a = gpu.get_field(c, cell_centered=False).astype(np.float64)
        b = o64.field(c)
        num += float(np.sum((a - b) ** 2))
        den += float(np.sum(b ** 2))
    got = flux[0].get_flux_spectrum()
    expected = o64.flux_spectrum(0)
    out["error"] = {"mirror80_600_steps": {
        "fields_rel_l2_vs_f64": float(math.sqrt(num / den)),
        "flux_rel_vs_f64": float(np.max(np.abs(got - expected)) / np.max(np.abs(expected)))}}
    gpu.close()
    return out


def validate(device):
    """Relative errors of the float32 engine against the float64 oracle, bounded samples."""
    from meep_gpu_gb300 import FdtdDriver, workloads
    from oracle.oracle import Oracle, problem_from_driver
    out = {}
    steps = 600
    gpu, flux, _ = workloads.build("sphere80", FdtdDriver)
    gpu.run(num_steps=steps, progress_interval=steps)
    ref, _, _ = workloads.build("sphere80", FdtdDriver)
    o64 = Oracle(problem_from_driver(ref), "f64")
    o64.run(steps)
    num = den = 0.0
    for c in ("Ex", "Ey", "Ez", "Hx", "Hy", "Hz"):
        a = gpu.get_field(c, cell_centered=False).astype(np.float64)
        b = o64.field(c)
        num += float(np.sum((a - b) ** 2))
        den += float(np.sum(b ** 2))
    got = flux[0].get_flux_spectrum()
    expected = o64.flux_spectrum(0)
    out["sphere80_600_steps"] = {
        "fields_rel_l2_vs_f64": float(math.sqrt(num / den)),
        "flux_rel_vs_f64": float(np.max(np.abs(got - expected)) / np.max(np.abs(expected)))}
    gpu.close()
    out["sphere192_8dft_600_steps"] = headline_error(600)
    return out


def headline_error(steps: int) -> dict:
    """The timed workload's own error: the 192^3 eight-DFT case after ``steps`` steps
    against the float64 oracle (fields relative L2 over E and H; each flux plane's
    largest deviation relative to its peak; each DFT volume's relative L2)."""
    from meep_gpu_gb300 import FdtdDriver, workloads
    from oracle.oracle import Oracle, problem_from_driver

    os.environ.setdefault("OMP_NUM_THREADS", str(cpu_threads()))
    gpu, flux, dft = workloads.build("sphere192_8dft", FdtdDriver)
    gpu.run(num_steps=steps, progress_interval=steps)
    ref, _, _ = workloads.build("sphere192_8dft", FdtdDriver)
    t0 = time.perf_counter()
    o64 = Oracle(problem_from_driver(ref), "f64")
    o64.run(steps)
    oracle_s = time.perf_counter() - t0
    num = den = 0.0
    for c in ("Ex", "Ey", "Ez", "Hx", "Hy", "Hz"):
        a = gpu.get_field(c, cell_centered=False).astype(np.float64)
        b = o64.field(c)
        num += float(np.sum((a - b) ** 2))
        den += float(np.sum(b ** 2))
    flux_err = []
    for index, monitor in enumerate(flux):
        expected = o64.flux_spectrum(index)
        flux_err.append(float(np.max(np.abs(monitor.get_flux_spectrum() - expected)) / np.max(np.abs(expected))))
    dft_err = []
    for index, monitor in enumerate(dft):
        n2 = d2 = 0.0
        for c in monitor.components:
            expected = o64.dft(len(flux) + index, c)
            got = monitor.raw(c).reshape(expected.shape).astype(np.complex128)
            n2 += float(np.sum(np.abs(got - expected) ** 2))
            d2 += float(np.sum(np.abs(expected) ** 2))
        dft_err.append(float(math.sqrt(n2 / d2)) if d2 > 0 else 0.0)
    gpu.close()
    return {"fields_rel_l2_vs_f64": float(math.sqrt(num / den)), "flux_rel_vs_f64_max": max(flux_err),
            "flux_rel_vs_f64": flux_err, "dft_rel_l2_vs_f64": dft_err,
            "oracle_seconds": round(oracle_s, 1), "oracle_threads": cpu_threads()}


if __name__ == "__main__":
    main()
