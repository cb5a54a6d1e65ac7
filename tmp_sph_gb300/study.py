"""Accuracy study of the resident solver's precisions on one dam-break case.

Runs the same seeded case in FP32, mixed precision and FP64 for `steps` steps, sampling the
surge front (largest fluid x) and a wall pressure probe every `every` steps on the GPU, and
reports the relative L2 difference of each precision's fields (displacement, velocity,
rho - rho0, p; fluid particles) at checkpoints and at the end, and of the time series, from the
FP64 run of the same solver.

    python -m tmp_sph_gb300.study --case precision --steps 5000 --every 50

prints one JSON object.  The default case is the 765,828-particle dam break (tank
1.0 x 0.5 x 0.6 m, water 0.4 x 0.5 x 0.3 m, dx 5 mm); the default probe is the wall pressure at
(1.0, 0.25, 0.05) m on the far wall.  Water-height gauges (the reference's H2 and H4 at
x = 2.228 and 0.582 m, y = 0.5 m, src/io/io.cu:236-256) are added with --gauges x y zmax ...:

    python -m tmp_sph_gb300.study --case obstacle --probe 2.31 0.5 0.03 \
        --gauges 2.228 0.5 0.4 0.582 0.5 0
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import api, cases
from . import solver as S


def rel_l2(a, b, floor=0.0) -> float:
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    den = max(float(np.linalg.norm(b)), floor)
    return float(np.linalg.norm(a - b)) / den if den > 0 else float(np.linalg.norm(a - b))


def run_precision(st, p, precision: str, steps: int, every: int, probe_xyz, stream,
                  checkpoints=(), gauges=()) -> dict:
    import torch
    n = len(st["rho"])
    probes = [(api.SPH_PROBE_FRONT, 0, 0, 0, 0, 0),
              (api.SPH_PROBE_PRESSURE, *probe_xyz, 0, 0)]
    # water-height gauges, 1.5 dx wide as the reference's (src/io/io.cu:239-252)
    probes += [(api.SPH_PROBE_HEIGHT, gx, gy, 0, 1.5 * float(p.dx), zmax)
               for gx, gy, zmax in gauges]
    series = {"t": [], "front_x": [], "wall_p": [], "kinetic": [], "potential": []}
    for g in range(len(gauges)):
        series[f"gauge_{g}"] = []
    with S.Solver(p, n, precision=precision) as sol:
        sol.upload(st["pos"], st["vel"], st["rho"], st["p"], st["type"], stream=stream)
        done = 0
        snaps = {}
        marks = sorted({c for c in checkpoints if 0 < c < steps})
        t0 = time.perf_counter()
        while True:
            if done in marks:
                snaps[done] = sol.download_f64(stream=stream)
            vals, stats = sol.probe(probes, stream=stream)
            series["t"].append(done * float(p.dt))
            series["front_x"].append(vals[0])
            series["wall_p"].append(vals[1])
            series["kinetic"].append(stats["kinetic"])
            series["potential"].append(stats["potential"])
            for g in range(len(gauges)):
                series[f"gauge_{g}"].append(vals[2 + g])
            if done >= steps:
                break
            k = min(every, steps - done)
            nxt = [c for c in marks if c > done]
            if nxt:
                k = min(k, nxt[0] - done)
            sol.step(k, stream=stream)
            done += k
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        out = sol.download_f64(stream=stream)
        flags = sol.error_flags(stream=stream)
        rebuilds = sol.rebuild_count(stream=stream)
    snaps[steps] = out
    return {"fields": out, "snaps": snaps, "series": series, "seconds": wall, "flags": flags,
            "rebuilds": rebuilds, "final_stats": stats}


def field_errors(a: dict, b: dict, st: dict) -> dict:
    fl = st["type"] == 1
    n_f = int(fl.sum())
    return {
        "disp": rel_l2(a["pos"][fl] - st["pos"][fl], b["pos"][fl] - st["pos"][fl]),
        "vel": rel_l2(a["vel"][fl], b["vel"][fl], floor=1e-3 * np.sqrt(n_f)),
        "drho": rel_l2(a["rho"][fl] - 1000.0, b["rho"][fl] - 1000.0),
        "p": rel_l2(a["p"][fl], b["p"][fl]),
    }


def compare(res: dict, ref: dict, st: dict) -> dict:
    out = {f"step_{k}": field_errors(res["snaps"][k], ref["snaps"][k], st)
           for k in sorted(res["snaps"]) if k in ref["snaps"]}
    sa, sb = res["series"], ref["series"]
    out["series"] = {k: rel_l2(sa[k], sb[k]) for k in sa
                     if k not in ("t", "potential") and k in sb}
    return out


def study(case: str, steps: int, every: int, probe_xyz, precisions, checkpoints=(),
          gauges=()) -> dict:
    import torch
    st, p = cases.build(case, physics="config")
    stream = torch.cuda.Stream()
    runs = {prec: run_precision(st, p, prec, steps, every, probe_xyz, stream, checkpoints,
                                gauges)
            for prec in precisions}
    ref = runs.get("fp64")
    report = {"case": case, "particles": len(st["rho"]), "fluid": int((st["type"] == 1).sum()),
              "steps": steps, "dt_s": float(p.dt), "sample_every": every,
              "wall_probe_m": list(probe_xyz), "gauges_m": [list(g) for g in gauges],
              "runs": {}}
    for prec, r in runs.items():
        entry = {"seconds": r["seconds"], "ms_per_step": 1e3 * r["seconds"] / max(1, steps),
                 "device_error_flags": r["flags"], "list_rebuilds": r["rebuilds"],
                 "final_front_x": r["series"]["front_x"][-1],
                 "final_wall_p": r["series"]["wall_p"][-1],
                 "max_wall_p": max(r["series"]["wall_p"])}
        if ref is not None and prec != "fp64":
            entry["rel_l2_vs_fp64"] = compare(r, ref, st)
        report["runs"][prec] = entry
    report["series"] = {prec: {k: v[:: max(1, len(v) // 50)] for k, v in r["series"].items()}
                        for prec, r in runs.items()}
    return report


def main(argv=None) -> None:
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--case", default="precision")
    ap.add_argument("--steps", type=int, default=5000)
    ap.add_argument("--every", type=int, default=50)
    ap.add_argument("--probe", type=float, nargs=3, default=(1.0, 0.25, 0.05))
    ap.add_argument("--precisions", nargs="+",
                    default=["fp64", "fp32", "mixed", "mixed_comp", "mixed_abs"])
    ap.add_argument("--compare-at", type=int, nargs="*", default=[1000],
                    help="also compare the fields after these step counts")
    ap.add_argument("--gauges", type=float, nargs="*", default=[],
                    help="water-height gauges as x y zmax triples (zmax 0: no cap)")
    ap.add_argument("--out", default=None, help="also write the JSON here")
    args = ap.parse_args(argv)
    if len(args.gauges) % 3:
        ap.error("--gauges takes x y zmax triples")
    gauges = [tuple(args.gauges[i:i + 3]) for i in range(0, len(args.gauges), 3)]
    rep = study(args.case, args.steps, args.every, tuple(args.probe), args.precisions,
                args.compare_at, gauges)
    text = json.dumps(rep)
    if args.out:
        with open(args.out, "w") as f:
            f.write(text)
    print(text, flush=True)


if __name__ == "__main__":
    main()
