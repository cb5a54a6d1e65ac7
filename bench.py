"""Benchmark of the SPH hot path on one GB300 (or N independent replicas under torchrun).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--case large] [--impl ours|reference]

A step is one full predictor-corrector step (two cell-list builds, four neighbour passes,
two integrator updates) of the 4,963,548-particle dam break (tank 1.0 x 0.5 x 0.6 m, water
0.4 x 0.5 x 0.3 m, dx 2.5 mm, +-0.01 dx seeded jitter, h = 1.3 dx, Tait EOS, plain FP32).
The timed loop replays the step as a CUDA graph with the state resident in HBM; the state
(~180 MB read and written per pass) is larger than the 129 MB L2, so no flush is needed.

Printed: one JSON line (rank 0) with
  value        particle-steps/s over all ranks (weak scaling: every rank runs its own replica)
  e2e          the same metric through sph_step_host (pinned host buffers, upload + step +
               download inside the timed region)
  roofline     the dominant kernel's algorithmic bytes per launch / its CUDA-event duration
  cpu_baseline the oracle (C restatement of the reference, OpenMP) on a bounded sample
  clocks       nvidia-smi SM clocks and throttle reasons sampled during the timed region

--impl reference times the reference's hot path on the host cores instead: the reference has
no CPU implementation of its own, so that is the oracle's restatement of it (all threads).
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

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle-steps/s"
UNIT = "particle-steps/s"

# Algorithmic bytes per particle and pass, FP32 state, each array read or written once
# (the reference's dataflow): hash 20, sort 16, permute 80, neighbour pass 1 52,
# neighbour pass 2 60, integrator 102 (mean of predictor 108 and corrector 96).
B_HASH, B_SORT, B_PERMUTE, B_PASS1, B_PASS2, B_INTEGRATE = 20, 16, 80, 52, 60, 102
# Phase -> algorithmic bytes per particle per launch of the fused kernels
PHASE_BYTES = {"sort": B_SORT, "gather_cells": B_PERMUTE, "nbr_build": 16, "pass1": B_PASS1,
               "pass2_integrate": B_PASS2 + B_INTEGRATE + B_HASH}
PHASE_KERNEL = {"sort": "k_rs_upsweep/k_rs_scan/k_rs_downsweep",
                "gather_cells": "k_gather + k_cell_mark/k_cell_fill",
                "nbr_build": "k_nbr_build (one cell walk; positions read once = 16 B)",
                "pass1": "k_pass1_g<2 lanes> (k_pass1 with one lane)",
                "pass2_integrate": "k_pass2<MODE_PRED|MODE_CORR>"}


def dist_env():
    from tmp_sph_gb300.replicas import dist_env as env
    return env()


PHASE_NCU_NAME = {"nbr_build": "k_nbr_build", "pass1": "k_pass1", "pass2_integrate": "k_pass2"}


def ncu_summary(key: str) -> dict:
    """A per-kernel figure from the committed ncu summary of this workload (a line
    `key: {json}`): traffic_bytes_per_launch (dram__bytes_read.sum + dram__bytes_write.sum),
    l1_data_pipe_pct (l1tex__data_pipe_lsu_wavefronts, % of peak)."""
    path = os.path.join(ROOT, "profiles", "neighbour_kernels_large.md")
    try:
        for line in open(path):
            if line.startswith(key + ":"):
                return json.loads(line.split(":", 1)[1])
    except (OSError, ValueError):
        pass
    return {}


def ncu_traffic() -> dict:
    return ncu_summary("traffic_bytes_per_launch")


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons every 200 ms while running."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_id: str):
        self.gpu_id = gpu_id
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", self.gpu_id, f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            time.sleep(0.3)
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self) -> dict:
        sm, mx, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": float(max(mx)) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def gpu_uuid(dev_index: int) -> str:
    import torch
    try:
        u = str(torch.cuda.get_device_properties(dev_index).uuid)
        return u if u.startswith("GPU-") else "GPU-" + u
    except Exception:
        return str(dev_index)


def build_case(name: str):
    from tmp_sph_gb300 import cases
    return cases.build(name, physics="config")


def count_launches(num_cells: int, half_steps: int, rebuilds: int, mode: str) -> int:
    """Kernels launched over `half_steps` half steps with `rebuilds` list rebuilds."""
    bits = 1
    while bits < 31 and (1 << bits) < num_cells:
        bits += 1
    passes = (bits + 7) // 8
    # every half step: rebuild decision, pass 1, pass 2; a rebuild adds the sort-totals
    # clear, 3 kernels per radix pass, gather + copy back, cell-start clear, mark and fill,
    # and the neighbour-list build.  In gated mode the rebuild kernels are launched every
    # half step (and return at once when the lists are kept).
    rebuild_kernels = 3 * passes + 7
    if mode == "gated":
        return half_steps * (3 + rebuild_kernels)
    return 3 * half_steps + rebuilds * rebuild_kernels


def cpu_baseline(st, p, budget_s: float = 20.0) -> dict:
    """The oracle (reference arithmetic, OpenMP over all host threads) on the full workload,
    as many whole steps as fit in about budget_s (at least one)."""
    from oracle import oracle as O
    threads = O.set_threads(0)
    P = O.params_like(p)
    n = len(st["rho"])
    t0 = time.perf_counter()
    O.run(P, st, 1)
    t1 = time.perf_counter()
    steps = 1
    one = t1 - t0
    extra = int(max(0, min(4, math.floor((budget_s - one) / max(one, 1e-9)))))
    if extra > 0:
        O.run(P, st, extra)
        steps += extra
    dt = time.perf_counter() - t0
    return {"value": n * steps / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{steps} full step(s) of the same {n}-particle workload "
                      f"(C restatement of the reference src/ step loop, float, OpenMP)"}


def run_reference(args):
    """The reference arm: the reference has no CPU implementation of its own, so this times the
    oracle's C restatement of its step loop (src/sph/sph_run.cu:285-336) on all host cores, on
    the same workload.  The inputs and parameters come from the oracle side (oracle/workload.py:
    its own generator and parameter derivation), so this process loads no product library.
    Under torchrun only rank 0 runs; the others exit at once."""
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if int(os.environ.get("RANK", "0")) != 0:
        return
    from oracle import oracle as O, workload as W
    if args.case not in W.GEOM:
        print(json.dumps({"impl": "reference", "unavailable":
                          f"case {args.case}: the reference arm runs the single-case workloads"}))
        return
    st, P = W.build(args.case)
    n = len(st["rho"])
    n_fluid = st["n_fluid"]
    threads = O.set_threads(0)
    # the same number of warm-up steps as the timed arm, within a bounded time
    t0 = time.perf_counter()
    warm = 0
    cur = st
    while warm < args.warmup and (warm == 0 or time.perf_counter() - t0 < args.ref_budget / 3):
        cur = O.run(P, cur, 1)
        warm += 1
    t0 = time.perf_counter()
    steps = 0
    while steps < args.steps and (steps == 0 or time.perf_counter() - t0 < args.ref_budget):
        cur = O.run(P, cur, 1)
        steps += 1
    dt = time.perf_counter() - t0
    val = n * steps / dt
    line = {
        "metric": METRIC, "value": val, "unit": UNIT, "impl": "reference", "n_gpus": ws,
        "steps": steps, "warmup": warm, "ms_per_step": 1e3 * dt / steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded dam-break generator, oracle side)",
        "config": config_block(args, P, n),
        "fluid_particle_steps_per_s": n_fluid * steps / dt,
        "cpu_baseline": {"value": val, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{steps} full step(s) of the {n}-particle workload after "
                                   f"{warm} warm-up step(s), on all {threads} host threads "
                                   f"(requested {args.steps}, capped at {args.ref_budget:.0f} s)"},
        "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def set_lanes(sol, args) -> None:
    """Lanes per particle of the two list passes: --lanes for both, else --pass1-lanes (0: the
    precision's default) and --pass2-lanes."""
    from tmp_sph_gb300 import api
    if args.lanes is not None:
        sol.set_option(api.SPH_OPT_LANES_PER_PARTICLE, args.lanes)
    else:
        sol.set_option(api.SPH_OPT_PASS1_LANES, args.pass1_lanes)
        sol.set_option(api.SPH_OPT_PASS2_LANES, args.pass2_lanes)


def set_subcell(sol, args) -> None:
    from tmp_sph_gb300 import api
    if args.subcell is not None:
        sol.set_option(api.SPH_OPT_SUBCELL_ORDER, args.subcell)


def lanes_in_effect(sol) -> dict:
    """Launch shape of the neighbour kernels in effect (defaults resolved)."""
    from tmp_sph_gb300 import api
    return {"lanes_per_particle_pass1_pass2": [sol.get_option(api.SPH_OPT_PASS1_LANES),
                                               sol.get_option(api.SPH_OPT_PASS2_LANES)],
            "block_threads": sol.get_option(api.SPH_OPT_BLOCK_THREADS),
            "subcell_order": sol.get_option(api.SPH_OPT_SUBCELL_ORDER)}


def config_block(args, p, n, lanes=None):
    return {"workload": f"dam_break_{args.case}_{getattr(args, 'precision', 'fp32')}", "particles": n,
            "fluid_particles": n - p.num_boundary, "dx_m": p.dx, "h_over_dx": 1.3,
            "cells": p.num_cells, "eos": "tait", "dt_s": p.dt,
            "parallelism": f"replicas x{int(os.environ.get('WORLD_SIZE', '1'))}",
            "l2": "state larger than L2 (no flush needed)",
            "neighbour_list_skin_over_kh": args.skin / 1000.0,
            "graph_mode": args.graph_mode, "pairs": args.pairs,
            **(lanes or {}), "adaptive_skin": args.adaptive_skin}


def run_batch(args):
    """--case batchN: N independent dam breaks (tank 1.0 x 0.5 x 0.6 m, dx 5 mm, water blocks of
    width U[0.2, 0.6] m and height U[0.15, 0.45] m) advanced together by one batched solver.
    Device-resident throughput only (all instances' particles per second)."""
    import torch
    import torch.distributed as dist
    from tmp_sph_gb300 import api, build, cases, replicas, solver as S
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    if ws > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    build.build()
    n_inst = int(args.case[5:] or 64)
    # weak scaling: every rank advances its own batch of n_inst instances (its own seed)
    states, p = cases.batch(n_inst, seed=20240611 + 1009 * rank)
    n = sum(len(st["rho"]) for st in states)
    stream = torch.cuda.Stream()
    tuned = None
    if args.autotune:
        from tmp_sph_gb300 import autotune
        tuned = autotune.tune(p, states, precision=args.precision)
        args.skin = tuned["skin_permille"]
    sol = S.Solver(p, n, precision=args.precision)
    sol.set_option(api.SPH_OPT_SKIN_PERMILLE, args.skin)
    sol.set_option(api.SPH_OPT_CONDITIONAL_GRAPH, int(args.graph_mode == "conditional"))
    sol.set_option(api.SPH_OPT_PAIRS, args.pairs)
    set_lanes(sol, args)
    set_subcell(sol, args)
    sol.set_option(api.SPH_OPT_ADAPTIVE_SKIN, args.adaptive_skin)
    if tuned:
        autotune.apply(sol, tuned)
    lanes = lanes_in_effect(sol)
    sol.upload_instances(states, stream=stream)
    sol.step(args.warmup, stream=stream)
    torch.cuda.synchronize()
    r0 = sol.rebuild_count(stream=stream)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(gpu_uuid(local)) as clk:
        replicas.barrier()
        torch.cuda.synchronize()
        ev0.record(stream)
        sol.step(args.steps, stream=stream)
        ev1.record(stream)
        torch.cuda.synchronize()
        replicas.barrier()
    ms = replicas.reduce_max(ev0.elapsed_time(ev1))
    n_job = int(replicas.reduce_sum(n))
    rebuilds = sol.rebuild_count(stream=stream) - r0
    flags = sol.error_flags(stream=stream)
    sol.close()
    fluid = [int((st["type"] == 1).sum()) for st in states]
    line = {
        "metric": METRIC, "value": n_job * args.steps / (ms / 1e3), "unit": UNIT, "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": {"fp32": "f32", "mixed": "f32+f64", "mixed_comp": "f32+f64",
                  "fp64": "f64"}[args.precision],
        "data": "synthetic (seeded dam-break generator)",
        "config": {"workload": f"dam_break_batch{n_inst}_{args.precision}",
                   "instances_per_gpu": n_inst, "particles": n_job, "particles_rank0": n,
                   "fluid_min": min(fluid), "fluid_max": max(fluid),
                   "parallelism": f"instances x{ws} (independent batches, no collective)",
                   "dx_m": p.dx, "dt_s": p.dt, "cs": p.cs,
                   "neighbour_list_skin_over_kh": args.skin / 1000.0,
                   "graph_mode": args.graph_mode,
                   **lanes},
        "list_rebuilds": {"timed": rebuilds, "half_steps": 2 * args.steps},
        "autotune": autotune.summary(tuned) if tuned else None,
        "gpu_launches": count_launches(sol_cells_batch(p, n_inst, args.skin), 2 * args.steps,
                                       rebuilds, args.graph_mode),
        "clocks": clk.summary(),
        "device_error_flags": flags,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        dist.destroy_process_group()


def sol_cells_batch(p, n_inst: int, skin: int) -> int:
    """Cells of the stacked grid of n_inst instances (for the launch count's key width)."""
    import math
    cell = max(float(p.kh) * (1.0 + skin / 1000.0), float(p.cell_size))
    dims = [max(1, math.ceil((p.grid_max[c] - p.grid_min[c]) / cell)) for c in range(3)]
    return dims[0] * dims[1] * n_inst * (dims[2] + 1)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--case", default="large")
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--ref-budget", type=float, default=150.0)
    ap.add_argument("--e2e-steps", type=int, default=20)
    ap.add_argument("--graph-mode", default="conditional", choices=["conditional", "gated"],
                    help="rebuild kernels of the step graph under conditional nodes, or launched "
                         "every half step and returning at once when the lists are kept")
    ap.add_argument("--precision", default="fp32", choices=["fp32", "mixed", "mixed_comp", "fp64"],
                    help="precision of the timed solver (the other two are timed beside it)")
    ap.add_argument("--autotune", action="store_true",
                    help="pick threads per block, particles per thread and skin with the "
                         "autotuner first (overrides --skin)")
    ap.add_argument("--pairs", type=int, default=0, choices=[0, 1],
                    help="two particles per thread over a union neighbour list (FP32, FP64)")
    ap.add_argument("--lanes", type=int, default=None, choices=[1, 2, 4, 8, 16],
                    help="lanes per particle in both neighbour-list passes")
    ap.add_argument("--pass1-lanes", type=int, default=0, choices=[0, 1, 2, 4, 8, 16],
                    help="lanes per particle in list pass 1 (0: 2 in FP32 with a skin, else 1)")
    ap.add_argument("--pass2-lanes", type=int, default=1, choices=[1, 2, 4, 8, 16],
                    help="lanes per particle in list pass 2")
    ap.add_argument("--adaptive-skin", type=int, default=1, choices=[0, 1],
                    help="lists take a skin up to --skin chosen at each rebuild (0: always --skin)")
    ap.add_argument("--subcell", type=int, default=None, choices=[0, 1, 2, 3],
                    help="order of the particles inside a cell (SPH_OPT_SUBCELL_ORDER; default: "
                         "the library's)")
    ap.add_argument("--skin", type=int, default=100,
                    help="neighbour-list skin in thousandths of kh (0: rebuild every half step)")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    if args.impl == "reference":
        return run_reference(args)
    if args.case.startswith("batch"):
        return run_batch(args)

    import torch
    import torch.distributed as dist
    from tmp_sph_gb300 import api, build, solver as S

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    if ws > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    build.build()
    st, p = build_case(args.case)
    n = len(st["rho"])
    stream = torch.cuda.Stream()
    tuned = None
    if args.autotune:
        from tmp_sph_gb300 import autotune
        tuned = autotune.tune(p, st, precision=args.precision)
        args.skin = tuned["skin_permille"]
    sol = S.Solver(p, n, precision=args.precision)
    sol.set_option(api.SPH_OPT_SKIN_PERMILLE, args.skin)
    sol.set_option(api.SPH_OPT_CONDITIONAL_GRAPH, int(args.graph_mode == "conditional"))
    sol.set_option(api.SPH_OPT_PAIRS, args.pairs)
    set_lanes(sol, args)
    set_subcell(sol, args)
    sol.set_option(api.SPH_OPT_ADAPTIVE_SKIN, args.adaptive_skin)
    if tuned:
        autotune.apply(sol, tuned)
    lanes = lanes_in_effect(sol)
    sol.upload(st["pos"], st["vel"], st["rho"], st["p"], st["type"], stream=stream)

    def barrier():
        if ws > 1:
            dist.barrier()

    with torch.cuda.stream(stream):
        sol.step(args.warmup, stream=stream)
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    rebuilds0 = sol.rebuild_count(stream=stream)
    sol_cells = sol.sorted_view()[3]
    with ClockSampler(gpu_uuid(local)) as clk:
        barrier()
        torch.cuda.synchronize()
        ev0.record(stream)
        sol.step(args.steps, stream=stream)
        ev1.record(stream)
        torch.cuda.synchronize()
        barrier()
    ms = ev0.elapsed_time(ev1)
    if ws > 1:
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    flags = sol.error_flags(stream=stream)
    rebuilds = sol.rebuild_count(stream=stream) - rebuilds0
    value = n * ws * args.steps / (ms / 1e3)

    # the same solver rebuilding its lists every half step (no skin): the cost a fast flow
    # approaches, for comparison with the reuse measured above
    k0 = min(args.steps, 50)
    sol.set_option(api.SPH_OPT_SKIN_PERMILLE, 0)
    sol.step(3, stream=stream)
    torch.cuda.synchronize()
    ev0.record(stream)
    sol.step(k0, stream=stream)
    ev1.record(stream)
    torch.cuda.synchronize()
    ms0 = ev0.elapsed_time(ev1)
    sol.set_option(api.SPH_OPT_SKIN_PERMILLE, args.skin)
    no_reuse = {"value": n * k0 / (ms0 / 1e3), "ms_per_step": ms0 / k0, "steps": k0}

    # the same workload in the other precisions of the solver (same skin, graph replay)
    def time_precision(precision: str, steps: int) -> dict:
        v = S.Solver(p, n, precision=precision)
        v.set_option(api.SPH_OPT_SKIN_PERMILLE, args.skin)
        set_lanes(v, args)
        set_subcell(v, args)
        v.set_option(api.SPH_OPT_ADAPTIVE_SKIN, args.adaptive_skin)
        v.upload(st["pos"], st["vel"], st["rho"], st["p"], st["type"], stream=stream)
        v.step(3, stream=stream)
        torch.cuda.synchronize()
        r0 = v.rebuild_count(stream=stream)
        ev0.record(stream)
        v.step(steps, stream=stream)
        ev1.record(stream)
        torch.cuda.synchronize()
        t = ev0.elapsed_time(ev1)
        out = {"value": n * steps / (t / 1e3), "ms_per_step": t / steps, "steps": steps,
               "list_rebuilds": v.rebuild_count(stream=stream) - r0,
               "device_error_flags": v.error_flags(stream=stream)}
        v.close()
        return out

    variants = {prec: time_precision(prec, min(args.steps, 10 if prec == "fp64" else 50))
                for prec in ("fp32", "mixed", "mixed_comp", "fp64") if prec != args.precision}

    # per-kernel device time from CUDA events around every phase, same stream
    prof_steps = min(args.steps, 20)
    sol.set_option(api.SPH_OPT_PROFILE, 1)
    sol.profile(reset=True)
    sol.step(prof_steps, stream=stream)
    prof = sol.profile(reset=True)
    sol.set_option(api.SPH_OPT_PROFILE, 0)
    flags |= sol.error_flags(stream=stream)
    hbm_peak, peak_kind = peaks()
    phases = {}
    for name, v in prof.items():
        per_launch_ms = v["ms"] / max(1, v["launches"])
        ach = PHASE_BYTES[name] * n / (per_launch_ms / 1e3) / 1e9
        phases[name] = {"ms_per_launch": per_launch_ms, "algorithmic_gbs": ach,
                        "share": v["ms"] / max(1e-9, sum(x["ms"] for x in prof.values())),
                        "kernels": PHASE_KERNEL[name]}
    dom = max(phases, key=lambda k: phases[k]["ms_per_launch"])
    traffic = ncu_traffic().get(PHASE_NCU_NAME.get(dom, ""))
    dom_ms = phases[dom]["ms_per_launch"]
    roof = {"bound": "hbm", "kernel": PHASE_KERNEL[dom],
            "achieved": phases[dom]["algorithmic_gbs"], "peak": hbm_peak, "unit": "GB/s",
            "frac": phases[dom]["algorithmic_gbs"] / hbm_peak, "peak_kind": peak_kind,
            "traffic": traffic,
            "traffic_source": "profiles/neighbour_kernels_large.md (ncu, one launch)",
            "dram_gbs_at_traffic": (traffic / (dom_ms / 1e3) / 1e9) if traffic else None,
            "bytes_per_particle": PHASE_BYTES[dom],
            "l1_data_pipe_pct": ncu_summary("l1_data_pipe_pct").get(PHASE_NCU_NAME.get(dom, "")),
            "note": "the neighbour kernels are issue- or L1-throughput bound (sparse gather "
                    "of neighbour data), not HBM bound; frac is algorithmic bytes over the "
                    "measured copy bandwidth"}

    # end to end through the C ABI with pinned host buffers
    hst = {k: torch.from_numpy(np.ascontiguousarray(st[k])).pin_memory()
           for k in ("pos", "vel", "rho", "p", "type")}
    hnp = {k: v.numpy() for k, v in hst.items()}
    e2e_sol = sol
    e2e_sol.set_option(api.SPH_OPT_USE_GRAPH, 1)
    e2e_sol.step_host(hnp, 1, stream=stream)  # warm
    for k in hst:
        hnp[k][...] = st[k]
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.e2e_steps):
        e2e_sol.step_host(hnp, 1, stream=stream)
    e2e_s = time.perf_counter() - t0
    barrier()
    e2e_val = n * ws * args.e2e_steps / e2e_s
    h2d = n * (12 + 12 + 4 + 4 + 4)
    d2h = n * (12 + 12 + 4 + 4)

    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(st, p)

    b_alg = 2 * (B_HASH + B_SORT + B_PERMUTE + B_PASS1 + B_PASS2 + B_INTEGRATE) + 48.0 * p.num_cells / n
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": {"fp32": "f32", "mixed": "f32+f64", "mixed_comp": "f32+f64",
                  "fp64": "f64"}[args.precision],
        "data": "synthetic (seeded dam-break generator)",
        "config": config_block(args, p, n, lanes),
        "hbm_gbs_algorithmic": value / ws * b_alg / 1e9,
        "hbm_frac_step_algorithmic": value / ws * b_alg / 1e9 / hbm_peak,
        "bytes_per_particle_step": b_alg,
        "roofline": roof,
        "phases": phases,
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_val, "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "steps": args.e2e_steps},
        "gpu_launches": count_launches(sol_cells, 2 * args.steps, rebuilds, args.graph_mode),
        "list_rebuilds": {"timed": rebuilds, "half_steps": 2 * args.steps,
                          "skin_permille": args.skin},
        "rebuild_every_half_step": no_reuse,
        "autotune": autotune.summary(tuned) if tuned else None,
        "precision_variants": variants,
        "clocks": clk.summary(),
        "device_error_flags": flags,
    }
    sol.close()
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
