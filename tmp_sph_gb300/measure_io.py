"""Cost of the components either side of the step, on the GPU at hand.

    python -m tmp_sph_gb300.measure_io [--case large] [--out file.json]

prints one JSON object with

* generator and .dat files (the reference's `ini_fluid` inputs, src/io/io.cu:10-111):
  seconds to generate the case, to write its seven text files and to read them back;
* probes (src/io/io.cu:236-279): device time of one `sph_probe_read` with a surge front, two
  pressure probes and two water-height gauges plus the FP64 reductions, against one step;
* snapshots (src/sph/sph_run.cu:258-281): step time with an asynchronous snapshot of the
  whole state every 1 / 10 steps against none (the copy runs on a second stream), and the time
  of the legacy-VTK writer for one frame (binary and ASCII);
* escaped particles (src/sph/sph_run.cu:437-447): step time of a case whose escape box cuts
  the water column, with parked particles kept in the neighbour search at the parking point
  (the reference's behaviour) and taken out of it (`park_inactive`).
"""
from __future__ import annotations

import argparse
import json
import os
import tempfile
import time

import numpy as np

from . import api, cases
from . import solver as S
from .output import write_vtk


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
    t0 = time.perf_counter()
    st, p = cases.build(case, physics="config")
    t_gen = time.perf_counter() - t0
    n = len(st["rho"])
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
    import torch
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


def main(argv=None) -> None:
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--case", default="large")
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--out", default=None)
    args = ap.parse_args(argv)
    rep = {"files": measure_files(args.case), "solver": measure_solver(args.case, args.steps),
           "parking": measure_parking(args.steps)}
    text = json.dumps(rep)
    if args.out:
        with open(args.out, "w") as f:
            f.write(text)
    print(text, flush=True)


if __name__ == "__main__":
    main()
