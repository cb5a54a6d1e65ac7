"""Time the reference solver's own CUDA step loops on this GPU.  TEST INFRASTRUCTURE.

Runs each of the reference's code trees — the baseline src/ and the optimisation snapshots
opt_src_v0..v4 — from its fatbin (oracle/_ref, launched by oracle/ref_harness.cu with the
reference's own launch shapes and thrust::sort_by_key) on the same seeded workload as bench.py
and prints one JSON line per version: particle-steps/s by CUDA events on the default stream,
plus the relative L2 of its fluid velocity and density perturbation after the timed steps
against the baseline src/ run (v4's half-precision distance test is inexact at these spacings).

    python -m oracle.ref_cuda_bench [--case large] [--steps 10] [--warmup 2] [--versions src,v0,...]
"""
from __future__ import annotations

import argparse
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--case", default="large")
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=2)
    ap.add_argument("--physics", default="config")
    ap.add_argument("--versions", default="src,v0,v1,v2,v3,v4")
    args = ap.parse_args()
    import torch
    from tmp_sph_gb300 import cases
    from oracle import oracle as O
    from oracle.ref_harness import RefHarness
    cuda = torch.device("cuda:0")
    st, p = cases.build(args.case, physics=args.physics)
    P = O.params_like(p)
    P.eos = 0  # the reference kernels implement only the linear EOS
    n = len(st["rho"])
    fl = st["type"] == 1
    base = None
    for v in args.versions.split(","):
        H = RefHarness(v)
        H.set_params(P, n)
        d, s, w, tmp = H.alloc(st, cuda)
        H.init_ids(d)
        H.step(d, s, w, tmp, args.warmup)
        H.sync()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(torch.cuda.default_stream())
        H.step(d, s, w, tmp, args.steps)
        e1.record(torch.cuda.default_stream())
        H.sync()
        ms = e0.elapsed_time(e1)
        out = H.state(d, s)
        res = {"impl": f"reference_cuda_{v}", "case": args.case, "physics": args.physics,
               "particles": n, "steps": args.steps, "warmup": args.warmup,
               "ms_per_step": ms / args.steps,
               "particle_steps_per_s": n * args.steps / (ms / 1e3),
               "finite": bool(np.isfinite(out["vel"]).all())}
        if base is None:
            base, base_name = out, v
        else:
            res[f"vel_rel_l2_vs_{base_name}"] = rel(out["vel"][fl], base["vel"][fl])
            res[f"drho_rel_l2_vs_{base_name}"] = rel(out["rho"][fl] - 1000.0,
                                                     base["rho"][fl] - 1000.0)
        print(json.dumps(res), flush=True)
        del d, s, w, tmp
        torch.cuda.empty_cache()


if __name__ == "__main__":
    main()
