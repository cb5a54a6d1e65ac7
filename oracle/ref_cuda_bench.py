"""Time the reference solver's own CUDA step loop on this GPU.  TEST INFRASTRUCTURE.

Runs the reference's src/ kernels (oracle/_ref/ref_src.fatbin through oracle/ref_harness.cu:
calcHash, thrust::sort_by_key, reorder, both neighbour kernels, PC_prediction, recover, then
the same for PC_correction — src/sph/sph_run.cu:285-336) on the same seeded workload as
bench.py, with the reference's own constants (h = 1.5 dx, linear EOS, cs 25) or the
benchmark's (h = 1.3 dx; only the neighbour count differs for the timing), and prints one
JSON line with particle-steps/s measured by CUDA events on the default stream.

    python -m oracle.ref_cuda_bench [--case large] [--steps 10] [--warmup 2] [--physics config]
"""
from __future__ import annotations

import argparse
import json
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--case", default="large")
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=2)
    ap.add_argument("--physics", default="config")
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
    H = RefHarness()
    H.set_params(P, n)
    d, s, w, tmp = H.alloc(st, cuda)
    H.step(d, s, w, tmp, args.warmup)
    H.sync()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(torch.cuda.default_stream())
    H.step(d, s, w, tmp, args.steps)
    e1.record(torch.cuda.default_stream())
    H.sync()
    ms = e0.elapsed_time(e1)
    out = {"impl": "reference_cuda_src", "case": args.case, "physics": args.physics,
           "particles": n, "steps": args.steps, "ms_per_step": ms / args.steps,
           "particle_steps_per_s": n * args.steps / (ms / 1e3),
           "finite": bool(torch.isfinite(d["vel"]).all().item())}
    print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
