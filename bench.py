"""Benchmark of the SPH hot path on one GB300 (or N independent replicas under torchrun).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--case large] [--impl ours|reference]

A step is one full predictor-corrector step (two cell-list builds, four neighbour passes,
two integrator updates) of the 4,963,548-particle dam break (tank 1.0 x 0.5 x 0.6 m, water
0.4 x 0.5 x 0.3 m, dx 2.5 mm, +-0.01 dx seeded jitter, h = 1.3 dx, Tait EOS, plain FP32).
The timed loop replays the step as a CUDA graph with the state resident in HBM; the state
(~180 MB read and written per pass) is larger than the 129 MB L2, so no flush is needed.

Printed: one JSON line (rank 0) with
  value          particle-steps/s over all ranks (weak scaling: every rank runs its own
                 replica); fluid_particle_steps_per_s counts fluid particles only
  e2e            the same metric through sph_step_host (pinned host buffers, upload + step +
                 download inside the timed region)
  roofline       the dominant kernel's algorithmic bytes per launch / its CUDA-event duration,
                 with the DRAM traffic of a committed ncu capture at the same launch shape
  roofline_fp32  flops of the evaluated pairs per step (counted from the pair algebra, pair
                 counts of the initial state) / step time, over the FP32 FMA peak measured now
  configured_run the configured 1000 steps from rest, all timed, then the developed flow,
                 each with the list skin at its end, and the developed flow's device time
                 per phase (phase_ms_per_step)
  batched        the 64-instance batch: dam breaks of uneven size in one batched
                 mixed-precision solver
                 (graph replay; FP64 integration, FP32 sums on FP32 positions by default,
                 --batch-precision), beside the plain FP32 single-instance value above, and
                 the same batch in FP32 and in the other mixed form (short windows)
  drop_in_step_loop  the reference's own step loop through the library's C-ABI drop-ins
                 (calcHash ... recover every half step, on the reference grid)
  reference_cuda the reference's own CUDA versions (opt_src_v4, the best, and src/) on the
                 same state and GPU, from kernels compiled out of its sources (oracle/_ref)
  cpu_baseline   the oracle (C restatement of the reference, OpenMP) on a bounded sample
  clocks         nvidia-smi SM clocks and throttle reasons sampled during the timed region

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
                "pass1": "k_pass1 (k_pass1_g with two or four lanes)",
                "pass2_integrate": "k_pass2<MODE_PRED|MODE_CORR>"}


def dist_env():
    from tmp_sph_gb300.replicas import dist_env as env
    return env()


PHASE_NCU_NAME = {"nbr_build": "k_nbr_build", "pass1": "k_pass1", "pass2_integrate": "k_pass2"}
PROFILE_JSON = os.path.join(ROOT, "profiles", "neighbour_kernels.json")


def ncu_capture(phase: str, workload: str, shape: dict) -> dict:
    """The committed ncu capture of a phase's kernel (profiles/neighbour_kernels.json: one
    record per capture with the kernel, workload and launch shape it was taken at, its DRAM
    bytes per launch and L1 data-pipe utilisation).  Only a capture taken at the launch shape
    in effect describes the timed kernel; otherwise the result says why there is none."""
    name = PHASE_NCU_NAME.get(phase)
    if not name:
        return {"reason": f"no ncu capture is kept for phase {phase}"}
    try:
        with open(PROFILE_JSON) as f:
            caps = json.load(f)["captures"]
    except (OSError, ValueError, KeyError):
        return {"reason": "profiles/neighbour_kernels.json missing"}
    seen = []
    for c in caps:
        if not c.get("kernel", "").startswith(name) or c.get("workload") != workload:
            continue
        cshape = {k: c.get(k) for k in shape}
        if cshape == shape:
            return c
        seen.append(cshape)
    return {"reason": f"no capture of {name} on {workload} at {shape} (captured: {seen})"}


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


def count_launches(num_cells: int, half_steps: int, rebuilds: int, mode: str,
                   keep_keys: bool = False) -> int:
    """Kernels launched over `half_steps` half steps with `rebuilds` list rebuilds
    (keep_keys: a batch with per-instance decisions, one more kernel per rebuild)."""
    bits = 1
    while bits < 31 and (1 << bits) < num_cells:
        bits += 1
    passes = (bits + 7) // 8
    # every half step: rebuild decision, pass 1, pass 2; a rebuild adds the sort-totals
    # clear, 3 kernels per radix pass, gather + copy back, cell-start clear, mark and fill,
    # and the neighbour-list build.  In gated mode the rebuild kernels are launched every
    # half step (and return at once when the lists are kept).
    rebuild_kernels = 3 * passes + 7 + (1 if keep_keys else 0)
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


# Flops of one evaluated pair, counted from the pair algebra of the kernels
# (tmp_sph_gb300/csrc/equation/ns_pair.cuh, Pass1Acc::pair and Pass2Acc::pair; the reference's
# form is src/equation/ns.cu:99-108 and :206-248).  A fused multiply-add counts 2, a square
# root or reciprocal 1; the relative position and squared distance (8) are included.
FLOPS_P1_FLUID = 28   # pass 1, fluid i and fluid j: velocity-divergence term
FLOPS_P1_WALL = 24    # pass 1, boundary i and fluid j: pressure-extrapolation sums
FLOPS_P2_FLUID = 45   # pass 2, fluid i and fluid j: continuity, diffusion, pressure, damper, AV
FLOPS_P2_WALL = 41    # pass 2, fluid i and boundary j (no damper, no viscosity)
FLOPS_PARTICLE = 35   # per fluid particle and half step: sums to rates, integrator, EOS, hash


def pair_counts(st: dict, kh: float, sample: int = 200_000, seed: int = 7) -> dict:
    """Ordered pairs closer than kh in the state (the pairs the passes evaluate): fluid-fluid
    and fluid-boundary, estimated from a seeded sample of fluid particles with k-d trees."""
    from scipy.spatial import cKDTree
    pos = np.asarray(st["pos"], np.float64)
    fl = np.asarray(st["type"]) == 1
    F, B = pos[fl], pos[~fl]
    rng = np.random.default_rng(seed)
    sel = F[rng.choice(len(F), min(sample, len(F)), replace=False)]
    ff = (cKDTree(F).query_ball_point(sel, kh, return_length=True) - 1).mean()
    fb = cKDTree(B).query_ball_point(sel, kh, return_length=True).mean() if len(B) else 0.0
    return {"fluid": int(fl.sum()), "ff_pairs": float(ff * len(F)), "fb_pairs": float(fb * len(F)),
            "ff_per_fluid": float(ff), "fb_per_fluid": float(fb), "sample": len(sel)}


def flops_per_step(pc: dict) -> float:
    """Algorithmic FP32 flops of one full step (two half steps) for the pair counts pc."""
    half = (pc["ff_pairs"] * (FLOPS_P1_FLUID + FLOPS_P2_FLUID) + pc["fb_pairs"] * FLOPS_P1_WALL
            + pc["fb_pairs"] * FLOPS_P2_WALL + pc["fluid"] * FLOPS_PARTICLE)
    return 2.0 * half


def fp32_peak(stream) -> dict:
    """FP32 FMA throughput of this GPU, measured now (sph_measure_fp32_peak, CUDA events)."""
    import ctypes as C
    import torch
    from tmp_sph_gb300 import api
    sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    blocks = sms * 8
    sink = torch.empty(blocks * 256, dtype=torch.float32, device="cuda")
    fl, ms = C.c_double(0), C.c_double(0)
    api.call("sph_measure_fp32_peak", C.c_void_p(sink.data_ptr()), blocks, 40000, C.byref(fl),
             C.byref(ms), C.c_void_p(stream.cuda_stream))
    return {"tflops": fl.value / (ms.value / 1e3) / 1e12, "ms": ms.value, "blocks": blocks,
            "how": "sph_measure_fp32_peak: 8 independent FMA chains per thread, CUDA events"}


def dropin_measure(st: dict, p, stream, steps: int = 10, warmup: int = 3) -> dict:
    """The reference's own step loop (src/sph/sph_run.cu:285-336: calcHash, sortParticles,
    reorder, SPH_NS_simpleversion, PC_prediction / PC_correction and recover every half step,
    on the reference's grid and AoS arrays) run through this library's C-ABI drop-ins on the
    same state: what the reference's driver gets by linking the library instead of its own
    kernels, timed by CUDA events on `stream`."""
    import torch
    from tmp_sph_gb300 import api, solver as S
    n = len(st["rho"])
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to("cuda")
    d = {k: dev(st[k]) for k in ("pos", "vel", "rho", "p", "type")}
    s = {k: torch.empty_like(v) for k, v in d.items()}
    h = torch.empty(n, dtype=torch.int32, device="cuda")
    idx = torch.empty_like(h)
    cs = torch.empty(p.num_cells, dtype=torch.int32, device="cuda")
    ce = torch.empty_like(cs)
    rdt, dofv = torch.zeros(n, device="cuda"), torch.zeros(n, device="cuda")
    vdt = torch.zeros((n, 3), device="cuda")
    tmp = (torch.zeros((n, 3), device="cuda"), torch.zeros((n, 3), device="cuda"),
           torch.zeros(n, device="cuda"))
    scratch = torch.empty(api.sort_scratch_bytes(n), dtype=torch.uint8, device="cuda")
    with S.Solver(p, n) as sol:  # sph_ns takes its constants from a context
        def half(k):
            S.calc_hash(p, d["pos"], h, idx, n, stream)
            S.sort_particles(h, idx, n, 32, scratch, stream)  # the shim's full-int sort
            S.reorder(p, d["pos"], d["vel"], d["rho"], d["p"], d["type"], None, s["pos"],
                      s["vel"], s["rho"], s["p"], s["type"], None, h, idx, cs, ce, n, stream)
            sol.ns(s["pos"], s["vel"], s["rho"], s["p"], s["type"], rdt, vdt, cs, ce, n, h, dofv,
                   stream=stream)
            pc = S.pc_prediction if k == 0 else S.pc_correction
            pc(p, s["pos"], s["vel"], s["rho"], s["p"], rdt, vdt, idx, *tmp, n, s["type"], stream)
            S.recover(d["pos"], d["vel"], d["rho"], d["p"], n, idx, d["type"], None, s["pos"],
                      s["vel"], s["rho"], s["p"], s["type"], None, stream)
        for _ in range(warmup):
            half(0)
            half(1)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(steps):
            half(0)
            half(1)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / steps
    return {"value": n / (ms / 1e3), "unit": UNIT, "ms_per_step": ms, "steps": steps,
            "warmup": warmup, "path": "calcHash, sortParticles (32-bit keys), reorder, "
            "SPH_NS_simpleversion (27-cell walks on the reference grid), PC_prediction / "
            "PC_correction, recover through the C ABI, every half step"}


def reference_cuda_leg(st: dict, p, versions=(("v4", 1, 10), ("src", 0, 2))) -> dict:
    """The reference's own CUDA step loops on this GPU, on the same state: its best version
    (opt_src_v4) and its baseline (src/), from the kernels compiled out of its sources
    (oracle/_ref, launched by oracle/ref_harness.cu with its launch shapes and thrust sort).
    A baseline leg like cpu_baseline: none of this library's code runs in it.  The reference
    kernels implement only the linear EOS, so they run the same geometry and constants with
    p = cs^2 (rho - rho0)."""
    import torch
    try:
        from oracle import oracle as O
        from oracle.ref_harness import RefHarness
    except Exception as e:  # noqa: BLE001
        return {"unavailable": f"harness not importable: {e}"}
    P = O.params_like(p)
    P.eos = 0
    n = len(st["rho"])
    out = {}
    cuda = torch.device("cuda", torch.cuda.current_device())
    for v, warm, steps in versions:
        try:
            H = RefHarness(v)
        except Exception as e:  # noqa: BLE001
            out[v] = {"unavailable": str(e).splitlines()[0][:200]}
            continue
        H.set_params(P, n)
        d, s_, w, tmp = H.alloc(st, cuda)
        H.init_ids(d)
        H.step(d, s_, w, tmp, warm)
        H.sync()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(torch.cuda.current_stream())
        H.step(d, s_, w, tmp, steps)
        e1.record(torch.cuda.current_stream())
        H.sync()
        ms = e0.elapsed_time(e1)
        out[v] = {"value": n * steps / (ms / 1e3), "unit": UNIT, "ms_per_step": ms / steps,
                  "steps": steps, "warmup": warm}
        del d, s_, w, tmp
        torch.cuda.empty_cache()
    out["note"] = ("reference kernels compiled from its sources for sm_103a, default stream, "
                   "CUDA events; linear EOS (the only form they implement)")
    return out


def graph_node_gap_us(stream, nodes: int = 64, replays: int = 50) -> float:
    """Device time per kernel node of a replayed CUDA graph whose nodes are a chain of tiny
    dependent kernels (one-element adds): the launch-to-launch cost a persistent kernel could
    save per launch it replaces."""
    import torch
    x = torch.zeros(1, device="cuda")
    g = torch.cuda.CUDAGraph()
    with torch.cuda.stream(stream):
        x.add_(1.0)
        torch.cuda.synchronize()
        with torch.cuda.graph(g, stream=stream):
            for _ in range(nodes):
                x.add_(1.0)
    g.replay()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    with torch.cuda.stream(stream):
        for _ in range(replays):
            g.replay()
    e1.record(stream)
    torch.cuda.synchronize()
    return 1e3 * e0.elapsed_time(e1) / (nodes * replays)


def time_run(sol, stream, steps: int) -> tuple[float, int]:
    """(milliseconds, list rebuilds) of `steps` steps on `stream`, by CUDA events."""
    import torch
    r0 = sol.rebuild_count(stream=stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    sol.step(steps, stream=stream)
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1), sol.rebuild_count(stream=stream) - r0


def configured_run(sol, stream, st, n: int, n_fluid: int, run_steps: int, steps: int) -> dict:
    """The configured run on a fresh solver `sol`: the initial state uploaded, all `run_steps`
    steps timed (the flow develops and the lists are rebuilt more often than in a short window
    from rest), then `steps` more steps of the developed flow timed alone."""
    from tmp_sph_gb300 import api
    sol.upload(st["pos"], st["vel"], st["rho"], st["p"], st["type"], stream=stream)
    ms, rb = time_run(sol, stream, run_steps)
    skin_run = sol.list_skin(stream=stream)
    ms2, rb2 = time_run(sol, stream, steps)
    skin_dev = sol.list_skin(stream=stream)
    # device time per phase over a window of the developed flow (kernels launched one by
    # one with events around every phase; the rebuild kernels of a half step that keeps its
    # lists return at once)
    k = min(steps, 50)
    sol.set_option(api.SPH_OPT_PROFILE, 1)
    sol.profile(reset=True)
    rb3 = sol.rebuild_count(stream=stream)
    sol.step(k, stream=stream)
    prof = sol.profile(reset=True)
    rb3 = sol.rebuild_count(stream=stream) - rb3
    sol.set_option(api.SPH_OPT_PROFILE, 0)
    phases = {name: v["ms"] / k for name, v in prof.items() if v["launches"]}
    return {"run": {"steps": run_steps, "ms_per_step": ms / run_steps,
                    "value": n * run_steps / (ms / 1e3),
                    "fluid_value": n_fluid * run_steps / (ms / 1e3),
                    "list_rebuilds": rb, "half_steps": 2 * run_steps,
                    "list_skin_over_kh_at_end": skin_run},
            "developed_flow": {"after_steps": run_steps, "steps": steps,
                               "ms_per_step": ms2 / steps, "value": n * steps / (ms2 / 1e3),
                               "fluid_value": n_fluid * steps / (ms2 / 1e3),
                               "list_rebuilds": rb2, "half_steps": 2 * steps,
                               "list_skin_over_kh_at_end": skin_dev,
                               "phase_ms_per_step": {"steps": k, "list_rebuilds": rb3,
                                                     **phases}},
            "device_error_flags": sol.error_flags(stream=stream)}


def set_lanes(sol, args) -> None:
    """Lanes per particle of list pass 1 (--pass1-lanes; 0: the precision's default), the cell
    size (--divisions; 0: the library's default) and the threads per block of the neighbour
    kernels (--threads; 0: the precision's default)."""
    from tmp_sph_gb300 import api
    sol.set_option(api.SPH_OPT_PASS1_LANES, args.pass1_lanes)
    if args.divisions:
        sol.set_option(api.SPH_OPT_CELL_DIVISIONS, args.divisions)
    sol.set_option(api.SPH_OPT_BLOCK_THREADS, args.threads)


def lanes_in_effect(sol) -> dict:
    """Launch shape of the neighbour kernels in effect (defaults resolved)."""
    from tmp_sph_gb300 import api
    return {"lanes_per_particle_pass1_pass2": [sol.get_option(api.SPH_OPT_PASS1_LANES), 1],
            "block_threads": sol.get_option(api.SPH_OPT_BLOCK_THREADS),
            "cell_divisions": sol.get_option(api.SPH_OPT_CELL_DIVISIONS)}


def config_block(args, p, n, lanes=None):
    return {"workload": f"dam_break_{args.case}_{getattr(args, 'precision', 'fp32')}", "particles": n,
            "fluid_particles": n - p.num_boundary, "dx_m": p.dx, "h_over_dx": 1.3,
            "cells": p.num_cells, "eos": "tait", "dt_s": p.dt,
            "parallelism": f"replicas x{int(os.environ.get('WORLD_SIZE', '1'))}",
            "l2": "state larger than L2 (no flush needed)",
            "neighbour_list_skin_over_kh": args.skin / 1000.0,
            "graph_mode": args.graph_mode,
            **(lanes or {}), "adaptive_skin": args.adaptive_skin}


def batch_measure(n_inst: int, precision: str, args, stream, steps: int, warmup: int,
                  run_steps: int = 0, ws: int = 1, rank: int = 0, clocks=None) -> dict:
    """The batched workload: n_inst independent dam breaks (tank 1.0 x 0.5 x 0.6 m, dx 5 mm, water
    blocks of width U[0.2, 0.6] m and height U[0.15, 0.45] m drawn from the seed) advanced together
    by one batched solver: every half step of all instances is the same few launches, replayed as
    one CUDA graph. With ws > 1 ranks the one batch is split by instance (contiguous blocks of about
    equal particle counts, replicas.partition) and each rank advances its share: no collective on
    the data path, strong scaling. `steps` timed after `warmup`, then, with run_steps, the
    configured run from rest (run_steps steps timed) continued into the developed flow."""
    import torch
    from tmp_sph_gb300 import api, cases, replicas, solver as S
    states, p = cases.batch(n_inst, seed=20240611)
    counts = [len(st["rho"]) for st in states]
    lo, hi = replicas.partition(counts, ws)[rank]
    mine = states[lo:hi]
    n = sum(counts[lo:hi])
    n_all = sum(counts)
    fluid = [int((st["type"] == 1).sum()) for st in states]
    n_fluid_all = sum(fluid)
    tuned = None
    skin = args.skin
    if args.autotune:
        from tmp_sph_gb300 import autotune
        tuned = autotune.tune(p, mine, precision=precision)
        skin = tuned["skin_permille"]
    def make_solver():
        v = S.Solver(p, n, precision=precision)
        v.set_option(api.SPH_OPT_SKIN_PERMILLE, skin)
        v.set_option(api.SPH_OPT_CONDITIONAL_GRAPH, int(args.graph_mode == "conditional"))
        set_lanes(v, args)
        v.set_option(api.SPH_OPT_ADAPTIVE_SKIN, args.adaptive_skin)
        v.set_option(api.SPH_OPT_INSTANCE_DECISIONS, args.instance_decisions)
        if tuned:
            from tmp_sph_gb300 import autotune
            autotune.apply(v, tuned)
        return v

    def instance_rebuilds(v) -> dict:
        c = v.instance_rebuild_counts(hi - lo, stream=stream)
        return {"min": int(c.min()), "mean": float(c.mean()), "max": int(c.max())}

    sol = make_solver()
    lanes = lanes_in_effect(sol)
    sol.upload_instances(mine, stream=stream)
    sol.step(warmup, stream=stream)
    torch.cuda.synchronize()
    r0 = sol.rebuild_count(stream=stream)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    clk = clocks if clocks is not None else _NoClock()
    with clk:
        replicas.barrier()
        torch.cuda.synchronize()
        ev0.record(stream)
        sol.step(steps, stream=stream)
        ev1.record(stream)
        torch.cuda.synchronize()
        replicas.barrier()
    ms = replicas.reduce_max(ev0.elapsed_time(ev1))
    rebuilds = sol.rebuild_count(stream=stream) - r0
    own = bool(sol.get_option(api.SPH_OPT_INSTANCE_DECISIONS)) and hi - lo > 1
    out = {"value": n_all * steps / (ms / 1e3), "unit": UNIT,
           "fluid_value": n_fluid_all * steps / (ms / 1e3), "ms_per_step": ms / steps,
           "steps": steps, "warmup": warmup,
           "dtype": {"fp32": "f32", "mixed": "f32+f64", "mixed_comp": "f32+f64",
                     "mixed_abs": "f32+f64", "fp64": "f64"}[precision],
           "config": {"workload": f"dam_break_batch{n_inst}_{precision}", "instances": n_inst,
                      "instances_this_rank": hi - lo, "particles": n_all,
                      "particles_this_rank": n, "fluid_particles": n_fluid_all,
                      "fluid_min": min(fluid), "fluid_max": max(fluid),
                      "parallelism": (f"instances split over {ws} ranks (no collective)"
                                      if ws > 1 else "one batched solver"),
                      "dx_m": p.dx, "dt_s": p.dt, "cs": p.cs,
                      "neighbour_list_skin_over_kh": skin / 1000.0,
                      "graph_mode": args.graph_mode, "instance_decisions": int(own), **lanes},
           "list_rebuilds": {"timed": rebuilds, "half_steps": 2 * steps},
           "gpu_launches": count_launches(
               sol_cells_batch(p, n_inst, skin, lanes["cell_divisions"]), 2 * steps,
               rebuilds, args.graph_mode, own),
           "autotune": None}
    if tuned:
        from tmp_sph_gb300 import autotune
        out["autotune"] = autotune.summary(tuned)
    flags = sol.error_flags(stream=stream)
    sol.close()
    if run_steps > 0 and tuned:
        # the library default over the same configured run, beside the autotuner's pick
        dsol = S.Solver(p, n, precision=precision)
        dsol.set_option(api.SPH_OPT_CONDITIONAL_GRAPH, int(args.graph_mode == "conditional"))
        dsol.upload_instances(mine, stream=stream)
        ms_d, rb_d = time_run(dsol, stream, run_steps)
        ms_d = replicas.reduce_max(ms_d)
        out["configured_run_default"] = {"steps": run_steps, "ms_per_step": ms_d / run_steps,
                                         "value": n_all * run_steps / (ms_d / 1e3),
                                         "list_rebuilds": rb_d, "half_steps": 2 * run_steps}
        flags |= dsol.error_flags(stream=stream)
        dsol.close()
    if run_steps > 0:
        sol = make_solver()
        sol.upload_instances(mine, stream=stream)
        ms_run, rb_run = time_run(sol, stream, run_steps)
        ms_run = replicas.reduce_max(ms_run)
        inst_rb = instance_rebuilds(sol)
        ms_dev, rb_dev = time_run(sol, stream, steps)
        ms_dev = replicas.reduce_max(ms_dev)
        out["configured_run"] = {"steps": run_steps, "ms_per_step": ms_run / run_steps,
                                 "value": n_all * run_steps / (ms_run / 1e3),
                                 "list_rebuilds": rb_run, "half_steps": 2 * run_steps,
                                 "instance_rebuilds": inst_rb}
        out["developed_flow"] = {"after_steps": run_steps, "steps": steps,
                                 "ms_per_step": ms_dev / steps,
                                 "value": n_all * steps / (ms_dev / 1e3),
                                 "list_rebuilds": rb_dev, "half_steps": 2 * steps}
        flags |= sol.error_flags(stream=stream)
        sol.close()
    out["device_error_flags"] = flags
    return out


class _NoClock:
    def __enter__(self):
        return self

    def __exit__(self, *a):
        return False

    def summary(self):
        return None


def run_batch(args):
    """--case batchN: the batched solver alone (batch_measure), one JSON line."""
    import torch
    import torch.distributed as dist
    from tmp_sph_gb300 import build
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    if ws > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    build.build()
    n_inst = int(args.case[5:] or 64)
    stream = torch.cuda.Stream()
    clk = ClockSampler(gpu_uuid(local))
    b = batch_measure(n_inst, args.precision, args, stream, args.steps, args.warmup,
                      run_steps=args.run_steps, ws=ws, rank=rank, clocks=clk)
    line = {"metric": METRIC, "value": b["value"], "unit": UNIT, "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": b["ms_per_step"],
            "higher_is_better": True, "scaling": "strong" if ws > 1 else "weak",
            "vs_baseline": None, "dtype": b["dtype"],
            "data": "synthetic (seeded dam-break generator)", "config": b["config"],
            **{k: v for k, v in b.items() if k not in ("value", "ms_per_step", "dtype", "config",
                                                      "steps", "warmup", "unit")},
            "clocks": clk.summary()}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        dist.destroy_process_group()


def sol_cells_batch(p, n_inst: int, skin: int, divisions: int = 1) -> int:
    """Cells of the stacked grid of n_inst instances (for the launch count's key width)."""
    import math
    cell = max(float(p.kh) * (1.0 + skin / 1000.0), float(p.cell_size)) / divisions
    dims = [max(1, math.ceil((p.grid_max[c] - p.grid_min[c]) / cell)) for c in range(3)]
    stride = (dims[2] + 2 * divisions - 1) // divisions * divisions
    return dims[0] * dims[1] * n_inst * stride


# ---------------------------------------------------------------- --components
# Cost of the components either side of the step (python bench.py --components [--case large]):
# * generator and .dat files (the reference's ini_fluid inputs, src/io/io.cu:10-111): seconds to
#   generate the case, to write its seven text files and to read them back;
# * probes (src/io/io.cu:236-279): one sph_probe_read with a surge front, two pressure probes
#   and two water-height gauges plus the FP64 reductions, against one step;
# * snapshots (src/sph/sph_run.cu:258-281): step time with an asynchronous snapshot of the
#   whole state every 1 / 10 steps against none (the copy runs on a second stream), and the
#   legacy-VTK writer for one frame (binary and ASCII);
# * escaped particles (src/sph/sph_run.cu:437-447): step time of a case whose escape box cuts
#   the water column, parked particles kept in the neighbour search (the reference's
#   behaviour) or taken out of it (park_inactive).

def _events():
    import torch
    return torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)


def step_ms(sol, stream, steps: int) -> float:
    import torch
    e0, e1 = _events()
    sol.step(2, stream=stream)
    torch.cuda.synchronize()
    e0.record(stream)
    sol.step(steps, stream=stream)
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / steps


def measure_files(case: str) -> dict:
    from tmp_sph_gb300 import api, cases
    t0 = time.perf_counter()
    st, p = cases.build(case, physics="config")
    t_gen = time.perf_counter() - t0
    n = len(st["rho"])
    import tempfile
    with tempfile.TemporaryDirectory() as d:
        t0 = time.perf_counter()
        api.write_dat(d, st)
        t_w = time.perf_counter() - t0
        size = sum(os.path.getsize(os.path.join(d, f)) for f in os.listdir(d))
        t0 = time.perf_counter()
        back = api.read_dat(d, n)
        t_r = time.perf_counter() - t0
    same = all(np.array_equal(back[k], st[k]) for k in ("pos", "vel", "rho", "p", "type"))
    return {"particles": n, "generate_s": t_gen, "write_dat_s": t_w, "read_dat_s": t_r,
            "dat_bytes": size, "round_trip_exact": bool(same)}


def measure_solver(case: str, steps: int) -> dict:
    import tempfile
    import torch
    from tmp_sph_gb300 import api, cases, solver as S
    from tmp_sph_gb300.output import write_vtk
    st, p = cases.build(case, physics="config")
    n = len(st["rho"])
    s = torch.cuda.Stream()
    out = {"particles": n}
    dx = float(p.dx)
    probes = [(api.SPH_PROBE_FRONT, 0, 0, 0, 0, 0),
              (api.SPH_PROBE_PRESSURE, 1.0, 0.25, 0.05, 0, 0),
              (api.SPH_PROBE_PRESSURE, 0.0, 0.25, 0.02, 0, 0),
              (api.SPH_PROBE_HEIGHT, 0.2, 0.25, 0, 1.5 * dx, 0),
              (api.SPH_PROBE_HEIGHT, 0.8, 0.25, 0, 1.5 * dx, 0)]
    with S.Solver(p, n) as sol:
        sol.upload(st["pos"], st["vel"], st["rho"], st["p"], st["type"], stream=s)
        base = step_ms(sol, s, steps)
        out["step_ms"] = base
        # probes: device time of the reduction launches (one read; the call synchronises)
        sol.probe(probes, stream=s)
        ts = []
        for _ in range(5):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            sol.probe(probes, stream=s)
            ts.append(time.perf_counter() - t0)
        out["probe_read_ms"] = 1e3 * float(np.median(ts))
        # snapshots on the copy stream while the steps continue
        host = {"pos": torch.empty((n, 3)).pin_memory(), "vel": torch.empty((n, 3)).pin_memory(),
                "p": torch.empty(n).pin_memory(), "type": torch.empty(n, dtype=torch.int32).pin_memory()}
        for every in (10, 1):
            e0, e1 = _events()
            torch.cuda.synchronize()
            e0.record(s)
            for k in range(steps):
                if k % every == 0:
                    api.call("sph_snapshot_begin", sol.handle, api.ptr(host["pos"]),
                             api.ptr(host["vel"]), None, api.ptr(host["p"]),
                             api.ptr(host["type"]), S._stream(s))
                sol.step(1, stream=s)
            e1.record(s)
            api.call("sph_snapshot_wait", sol.handle)
            torch.cuda.synchronize()
            out[f"step_ms_snapshot_every_{every}"] = e0.elapsed_time(e1) / steps
        out["snapshot_bytes"] = n * (12 + 12 + 4 + 4)
        h = {k: v.numpy() for k, v in host.items()}
        with tempfile.TemporaryDirectory() as d:
            for binary in (True, False):
                path = os.path.join(d, "f.vtk")
                t0 = time.perf_counter()
                write_vtk(path, h["pos"], h["vel"], h["p"], h["type"], binary=binary)
                dt = time.perf_counter() - t0
                key = "vtk_binary" if binary else "vtk_ascii"
                out[key + "_s"] = dt
                out[key + "_bytes"] = os.path.getsize(path)
    return out


def measure_parking(steps: int) -> dict:
    """The 765,828-particle case with the escape box's top at 0.28 m: the top 2 cm of the
    water column (about 32,000 particles) escapes in the first half step."""
    import torch
    from tmp_sph_gb300 import cases, solver as S
    st, p = cases.build("precision", physics="config")
    p.escape_max = type(p.escape_max)(p.escape_max[0], p.escape_max[1], 0.28)
    n = len(st["rho"])
    out = {"particles": n}
    for mode in (1, 0):
        p.park_inactive = mode
        s = torch.cuda.Stream()
        with S.Solver(p, n) as sol:
            sol.upload(st["pos"], st["vel"], st["rho"], st["p"], st["type"], stream=s)
            ms = step_ms(sol, s, steps)
            _, stats = sol.probe(stream=s)
            flags = sol.error_flags(stream=s)
        out[f"park_inactive_{mode}"] = {"step_ms": ms, "parked": stats["parked"],
                                        "device_error_flags": flags}
    return out


def run_components(args):
    import torch
    from tmp_sph_gb300 import build
    torch.cuda.set_device(0)
    build.build()
    steps = min(args.steps, 20)
    rep = {"components": True, "case": args.case, "files": measure_files(args.case),
           "solver": measure_solver(args.case, steps), "parking": measure_parking(steps)}
    print(json.dumps(rep), flush=True)


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
    ap.add_argument("--run-steps", type=int, default=1000,
                    help="steps of the configured run timed from rest (0: skip that block)")
    ap.add_argument("--batch-instances", type=int, default=64,
                    help="instances of the batched block of the default line (0: skip it)")
    ap.add_argument("--no-reference-cuda", action="store_true",
                    help="skip timing the reference's own CUDA versions")
    ap.add_argument("--components", action="store_true",
                    help="time the components either side of the step instead (generator, "
                         ".dat files, probes, snapshots, VTK writer, escaped particles)")
    ap.add_argument("--graph-mode", default="conditional", choices=["conditional", "gated"],
                    help="rebuild kernels of the step graph under conditional nodes, or launched "
                         "every half step and returning at once when the lists are kept")
    ap.add_argument("--precision", default="fp32",
                    choices=["fp32", "mixed", "mixed_comp", "mixed_abs", "fp64"],
                    help="precision of the timed solver (the other two are timed beside it)")
    ap.add_argument("--autotune", action="store_true",
                    help="pick threads per block, particles per thread and skin with the "
                         "autotuner first (overrides --skin)")
    ap.add_argument("--pass1-lanes", type=int, default=0, choices=[0, 1, 2, 4, 8, 16],
                    help="lanes per particle in list pass 1 (0: 2 in FP32 with a skin, else 1)")
    ap.add_argument("--threads", type=int, default=0,
                    help="threads per block of the neighbour kernels (SPH_OPT_BLOCK_THREADS; "
                         "0: the precision's default)")
    ap.add_argument("--divisions", type=int, default=0, choices=[0, 1, 2, 3],
                    help="cells per list cutoff (SPH_OPT_CELL_DIVISIONS; 0: the library's "
                         "default)")
    ap.add_argument("--batch-precision", default="mixed_abs",
                    choices=["mixed_abs", "mixed", "mixed_comp", "fp32"],
                    help="precision of the batched block of the default line: mixed_abs (FP64 "
                         "integration, FP32 sums on FP32 positions; the default) or mixed "
                         "(FP32 sums on cell-local offsets)")
    ap.add_argument("--instance-decisions", type=int, default=0, choices=[0, 1],
                    help="batches: 1 rebuilds each instance's lists on its own displacement "
                         "box and skin (SPH_OPT_INSTANCE_DECISIONS; 0, the default: one "
                         "decision for all)")
    ap.add_argument("--adaptive-skin", type=int, default=1, choices=[0, 1],
                    help="lists take a skin up to --skin chosen at each rebuild (0: always --skin)")
    ap.add_argument("--skin", type=int, default=100,
                    help="neighbour-list skin in thousandths of kh (0: rebuild every half step)")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    if args.impl == "reference":
        return run_reference(args)
    if args.case.startswith("batch"):
        return run_batch(args)
    if args.components:
        return run_components(args)

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
    n_fluid = int((st["type"] == 1).sum())
    stream = torch.cuda.Stream()
    tuned = None
    if args.autotune:
        from tmp_sph_gb300 import autotune
        tuned = autotune.tune(p, st, precision=args.precision)
        args.skin = tuned["skin_permille"]

    def configure(v):
        v.set_option(api.SPH_OPT_SKIN_PERMILLE, args.skin)
        v.set_option(api.SPH_OPT_CONDITIONAL_GRAPH, int(args.graph_mode == "conditional"))
        set_lanes(v, args)
        v.set_option(api.SPH_OPT_ADAPTIVE_SKIN, args.adaptive_skin)
        if tuned:
            from tmp_sph_gb300 import autotune
            autotune.apply(v, tuned)

    sol = S.Solver(p, n, precision=args.precision)
    configure(sol)
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
    skin_end = sol.list_skin(stream=stream)
    value = n * ws * args.steps / (ms / 1e3)

    # per-kernel device time from CUDA events around every phase, same stream
    prof_steps = min(args.steps, 20)
    sol.set_option(api.SPH_OPT_PROFILE, 1)
    sol.profile(reset=True)
    sol.step(prof_steps, stream=stream)
    prof = sol.profile(reset=True)
    sol.set_option(api.SPH_OPT_PROFILE, 0)
    flags |= sol.error_flags(stream=stream)

    # the same solver rebuilding its lists every half step (no skin): the cost a fast flow
    # approaches, for comparison with the reuse measured above
    k0 = min(args.steps, 50)
    sol.set_option(api.SPH_OPT_SKIN_PERMILLE, 0)
    sol.step(3, stream=stream)
    ms0, _ = time_run(sol, stream, k0)
    sol.set_option(api.SPH_OPT_SKIN_PERMILLE, args.skin)
    no_reuse = {"value": n * k0 / (ms0 / 1e3), "ms_per_step": ms0 / k0, "steps": k0}

    # the configured run (run_steps steps from rest, all timed) and the developed flow after it
    run = None
    if args.run_steps > 0:
        fresh = S.Solver(p, n, precision=args.precision)
        configure(fresh)
        run = configured_run(fresh, stream, st, n, n_fluid, args.run_steps, args.steps)
        fresh.close()
        flags |= run["device_error_flags"]
        if tuned:
            # the autotuner's pick against the library default over the same configured run
            fresh = S.Solver(p, n, precision=args.precision)
            fresh.set_option(api.SPH_OPT_CONDITIONAL_GRAPH, int(args.graph_mode == "conditional"))
            run["default"] = configured_run(fresh, stream, st, n, n_fluid, args.run_steps,
                                            args.steps)
            fresh.close()

    # the same workload in the other precisions of the solver (same skin, graph replay)
    def time_precision(precision: str, steps: int) -> dict:
        v = S.Solver(p, n, precision=precision)
        configure(v)
        v.upload(st["pos"], st["vel"], st["rho"], st["p"], st["type"], stream=stream)
        v.step(3, stream=stream)
        t, rb = time_run(v, stream, steps)
        out = {"value": n * steps / (t / 1e3), "ms_per_step": t / steps, "steps": steps,
               "list_rebuilds": rb, "device_error_flags": v.error_flags(stream=stream)}
        v.close()
        return out

    variants = {prec: time_precision(prec, min(args.steps, 10 if prec == "fp64" else 50))
                for prec in ("fp32", "mixed", "mixed_comp", "mixed_abs", "fp64")
                if prec != args.precision}

    hbm_peak, peak_kind = peaks()
    phases = {}
    for name, v in prof.items():
        per_launch_ms = v["ms"] / max(1, v["launches"])
        ach = PHASE_BYTES[name] * n / (per_launch_ms / 1e3) / 1e9
        phases[name] = {"ms_per_launch": per_launch_ms, "ms_per_step": v["ms"] / prof_steps,
                        "algorithmic_gbs": ach,
                        "share": v["ms"] / max(1e-9, sum(x["ms"] for x in prof.values())),
                        "kernels": PHASE_KERNEL[name]}
    lanes1 = lanes["lanes_per_particle_pass1_pass2"][0]
    if "pass1" in phases:
        phases["pass1"]["kernels"] = "k_pass1" if lanes1 == 1 else f"k_pass1_g<{lanes1} lanes>"
    dom = max(phases, key=lambda k: phases[k]["ms_per_launch"])
    dom_ms = phases[dom]["ms_per_launch"]
    workload = f"dam_break_{args.case}_{args.precision}"
    shape = {"block_threads": lanes["block_threads"],
             "lanes_pass1": lanes["lanes_per_particle_pass1_pass2"][0],
             "cell_divisions": lanes["cell_divisions"]}
    cap = ncu_capture(dom, workload, shape)
    traffic = cap.get("dram_bytes_per_launch")
    roof = {"bound": "hbm", "kernel": PHASE_KERNEL[dom],
            "achieved": phases[dom]["algorithmic_gbs"], "peak": hbm_peak, "unit": "GB/s",
            "frac": phases[dom]["algorithmic_gbs"] / hbm_peak, "peak_kind": peak_kind,
            "traffic": traffic,
            "traffic_source": ("profiles/neighbour_kernels.json: " + cap["kernel"] + " at "
                               + json.dumps(shape)) if traffic else cap.get("reason"),
            "dram_gbs_at_traffic": (traffic / (dom_ms / 1e3) / 1e9) if traffic else None,
            "bytes_per_particle": PHASE_BYTES[dom],
            "l1_data_pipe_pct": cap.get("l1_data_pipe_pct"),
            "note": "the neighbour kernels are bound by instruction issue and the latency "
                    "of their neighbour-record gathers (sparse gathers), not by HBM; frac is "
                    "algorithmic bytes over the measured copy bandwidth"}

    # FP32 arithmetic roofline: flops of the evaluated pairs (counted at the initial state)
    # over the FP32 FMA peak measured on this GPU now
    fp32 = None
    try:
        pc = pair_counts(st, float(p.kh))
        f_step = flops_per_step(pc)
        pk = fp32_peak(stream)
        ach = f_step * (value / ws / n) / 1e12
        fp32 = {"bound": "fp32", "achieved": ach, "peak": pk["tflops"], "unit": "TFLOP/s",
                "frac": ach / pk["tflops"], "peak_kind": "measured (this run)",
                "flops_per_step": f_step, "flops_per_particle_step": f_step / n,
                "pairs": pc, "peak_how": pk["how"],
                "flops_per_pair": {"pass1_fluid": FLOPS_P1_FLUID, "pass1_boundary": FLOPS_P1_WALL,
                                   "pass2_fluid": FLOPS_P2_FLUID, "pass2_boundary": FLOPS_P2_WALL,
                                   "per_fluid_particle_half_step": FLOPS_PARTICLE}}
    except Exception as e:  # noqa: BLE001
        fp32 = {"unavailable": str(e)[:200]}

    # end to end through the C ABI with pinned host buffers
    hst = {k: torch.from_numpy(np.ascontiguousarray(st[k])).pin_memory()
           for k in ("pos", "vel", "rho", "p", "type")}
    hnp = {k: v.numpy() for k, v in hst.items()}
    sol.set_option(api.SPH_OPT_USE_GRAPH, 1)
    sol.step_host(hnp, 1, stream=stream)  # warm
    for k in hst:
        hnp[k][...] = st[k]
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.e2e_steps):
        sol.step_host(hnp, 1, stream=stream)
    e2e_s = time.perf_counter() - t0
    barrier()
    e2e_val = n * ws * args.e2e_steps / e2e_s
    h2d = n * (12 + 12 + 4 + 4 + 4)
    d2h = n * (12 + 12 + 4 + 4)
    flags |= sol.error_flags(stream=stream)
    sol.close()

    # the batch comparison on one line: batched mixed precision (the 64-instance batch) against the
    # plain FP32 single-instance drop-in above
    batched = None
    if args.batch_instances > 0 and ws == 1:
        batched = batch_measure(args.batch_instances, args.batch_precision, args, stream,
                                args.steps, args.warmup, run_steps=args.run_steps,
                                clocks=ClockSampler(gpu_uuid(local)))
        batched["vs_plain_fp32"] = batched["value"] / value
        # what a persistent kernel could save: the graph's launch gaps (three kernel nodes per
        # half step that keeps its lists) against the step time
        gap = graph_node_gap_us(stream)
        batched["graph_node_gap_us"] = gap
        batched["launch_gap_share"] = 6 * gap / (1e3 * batched["ms_per_step"])
        batched["launch_gap_share_plain_fp32"] = 6 * gap / (1e3 * ms / args.steps)

    if args.batch_instances > 0 and ws == 1 and args.precision == "fp32":
        # the same batch in plain FP32 (what batching alone gives) and in the other mixed form
        # (cell-local offsets, or FP32 positions), short windows, beside the batched block
        other = "mixed" if args.batch_precision == "mixed_abs" else "mixed_abs"
        for prec in ("fp32", other):
            bf = batch_measure(args.batch_instances, prec, args, stream, args.steps, args.warmup)
            blk = {k: bf[k] for k in ("value", "ms_per_step", "steps", "device_error_flags")}
            blk["cell_divisions"] = bf["config"]["cell_divisions"]
            blk["vs_plain_fp32"] = bf["value"] / value
            batched[f"{prec}_same_batch"] = blk

    dropin = None
    if rank == 0 and ws == 1 and args.precision == "fp32":
        dropin = dropin_measure(st, p, stream)
        dropin["resident_over_dropin"] = value / dropin["value"]

    ref_cuda = None
    if rank == 0 and ws == 1 and not args.no_reference_cuda:
        ref_cuda = reference_cuda_leg(st, p)
        for v in ("v4", "src"):
            if isinstance(ref_cuda.get(v), dict) and "value" in ref_cuda[v]:
                ref_cuda[v]["this_over_reference"] = value / ref_cuda[v]["value"]
                if dropin:
                    dropin[f"over_reference_{v}"] = dropin["value"] / ref_cuda[v]["value"]

    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(st, p)

    b_alg = 2 * (B_HASH + B_SORT + B_PERMUTE + B_PASS1 + B_PASS2 + B_INTEGRATE) + 48.0 * p.num_cells / n
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": {"fp32": "f32", "mixed": "f32+f64", "mixed_comp": "f32+f64",
                  "mixed_abs": "f32+f64", "fp64": "f64"}[args.precision],
        "data": "synthetic (seeded dam-break generator)",
        "config": config_block(args, p, n, lanes),
        "fluid_particle_steps_per_s": n_fluid * ws * args.steps / (ms / 1e3),
        "hbm_gbs_algorithmic": value / ws * b_alg / 1e9,
        "hbm_frac_step_algorithmic": value / ws * b_alg / 1e9 / hbm_peak,
        "bytes_per_particle_step": b_alg,
        "roofline": roof,
        "roofline_fp32": fp32,
        "phases": phases,
        "cpu_baseline": cpu,
        "reference_cuda": ref_cuda,
        "drop_in_step_loop": dropin,
        "e2e": {"value": e2e_val, "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "steps": args.e2e_steps},
        "gpu_launches": count_launches(sol_cells, 2 * args.steps, rebuilds, args.graph_mode),
        "list_rebuilds": {"timed": rebuilds, "half_steps": 2 * args.steps,
                          "skin_permille": args.skin, "list_skin_over_kh_at_end": skin_end},
        "configured_run": run,
        "rebuild_every_half_step": no_reuse,
        "batched": batched,
        "autotune": autotune.summary(tuned) if tuned else None,
        "precision_variants": variants,
        "clocks": clk.summary(),
        "device_error_flags": flags,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
