"""Generate the golden fixtures that pin the CPU oracle to the reference.

Runs the reference solver's own kernels (src/, compiled from its sources into
oracle/_ref/ref_src.fatbin and launched by oracle/ref_harness.cu with the reference's launch
shapes, thrust::sort_by_key for the sort) on a GPU, on seeded inputs from the dam-break
generator, and stores inputs and outputs as compressed .npz files next to this script:

  ref_cells_<case>.npz  calcHash -> sortParticles -> reorder: hash (unsorted and sorted),
                        index, cellStart, cellEnd, gathered arrays
  ref_ns_<case>.npz     SPH_NS_simpleversion on the reorder output (perturbed velocities and
                        densities): densitydt, Veldt, dofv, rhop_sum, w_sum, wall p / rho
  ref_pc_<case>.npz     PC_prediction then PC_correction with given rates
  ref_run_<case>.npz    whole steps of the src step loop: state after 1 and after 5 steps

and, with --full-size, the fixtures of the full-size workloads:

  ref_cells_dam_4963548.json   calcHash -> sortParticles -> reorder of the reference on the
                           4,963,548-particle dam break (dx 2.5 mm, seeded jitter): SHA-256
                           digests of the input positions and of every output array (hash
                           unsorted and sorted, index, cellStart, cellEnd of the occupied cells,
                           the gathered arrays), with a few sampled values
  ref_run_dam_133968.npz      the reference's src step loop on the 133,968-particle dam break
                           (dx 1 cm, h = 1.3 dx, c0 = 24.26 m/s, delta 0.1, alpha 0.02,
                           dt = 0.25 h / c0, the reference's linear EOS): the fluid state after
                           200 steps

Usage (on a machine with a CUDA GPU and the fatbin):
    python tests/golden/make_golden.py [--full-size] [outdir]
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

# (name, case, dx, jitter, physics): small enough to keep each fixture at a few hundred kB
CASES = [
    ("tank_dx30", "small", 0.03, 0.01, "reference"),
    ("tank_tait_dx30", "small", 0.03, 0.01, "config"),
    ("refcase_dx50", "refcase", 0.05, 0.02, "reference"),
]


def gen_state(case, dx, jitter, physics):
    from tmp_sph_gb300 import cases
    st, p = cases.build(case, physics=physics, dx=dx, jitter=jitter, seed=12345)
    return st, p


def perturb(st, seed=7):
    rng = np.random.default_rng(seed)
    out = {k: v.copy() for k, v in st.items() if isinstance(v, np.ndarray)}
    fl = out["type"] == 1
    out["vel"][fl] = rng.uniform(-0.3, 0.3, (fl.sum(), 3)).astype(np.float32)
    out["rho"][fl] = (1000.0 * (1.0 + rng.uniform(0, 0.02, fl.sum()))).astype(np.float32)
    out["p"][fl] = (625.0 * (out["rho"][fl] - 1000.0)).astype(np.float32)
    return out


def params_arrays(P) -> dict:
    return {"param_" + k: np.asarray(v) for k, v in P.as_dict().items()}


def main(outdir=HERE):
    import torch
    from oracle import oracle as O
    from oracle.ref_harness import RefHarness
    cuda = torch.device("cuda:0")
    H = RefHarness()
    os.makedirs(outdir, exist_ok=True)
    for name, case, dx, jitter, physics in CASES:
        st, p = gen_state(case, dx, jitter, physics)
        P = O.params_like(p)
        n = len(st["rho"])
        if physics != "reference":
            # the reference kernels only know the linear EOS; Tait cases pin the cell list and
            # the neighbour pass on a Tait-consistent state (p given), not the integrator
            pass
        H.set_params(P, n)
        host = lambda t: t.detach().cpu().numpy()
        common = params_arrays(P)
        # ---- cell list
        d, s, w, tmp = H.alloc(perturb(st), cuda)
        H.calc_hash(d["pos"], w["hash"], w["index"])
        H.sync()
        hash_unsorted = host(w["hash"]).copy()
        H.sort(w["hash"], w["index"])
        H.reorder(d, s, w["hash"], w["index"], w["cs"], w["ce"])
        H.sync()
        pst = perturb(st)
        np.savez_compressed(
            os.path.join(outdir, f"ref_cells_{name}.npz"), **common,
            in_pos=pst["pos"], in_vel=pst["vel"], in_rho=pst["rho"], in_p=pst["p"], in_type=pst["type"],
            hash_unsorted=hash_unsorted, hash=host(w["hash"]), index=host(w["index"]),
            cell_start=host(w["cs"])[:P.num_cells], cell_end=host(w["ce"])[:P.num_cells],
            s_pos=host(s["pos"]), s_vel=host(s["vel"]), s_rho=host(s["rho"]), s_p=host(s["p"]),
            s_type=host(s["type"]))
        # ---- neighbour passes on the sorted, perturbed state
        H.ns(s, w, w["cs"], w["ce"], w["hash"])
        H.sync()
        np.savez_compressed(
            os.path.join(outdir, f"ref_ns_{name}.npz"),
            rho_dt=host(w["rho_dt"]), vel_dt=host(w["vel_dt"]), dofv=host(w["dofv"]),
            rhop_sum=host(w["rhop_sum"]), w_sum=host(w["w_sum"]), p_after=host(s["p"]),
            rho_after=host(s["rho"]))
        if physics == "reference":
            # ---- integrator with the rates just computed
            before = {k: host(s[k]).copy() for k in ("pos", "vel", "rho", "p")}
            H.pc(0, s, w, w["index"], tmp)
            H.sync()
            pred = {k: host(s[k]).copy() for k in ("pos", "vel", "rho", "p")}
            tmp_pred = {k: host(v).copy() for k, v in tmp.items()}
            H.pc(1, s, w, w["index"], tmp)
            H.sync()
            np.savez_compressed(
                os.path.join(outdir, f"ref_pc_{name}.npz"),
                **{"before_" + k: v for k, v in before.items()},
                **{"pred_" + k: v for k, v in pred.items()},
                **{"tmp_" + k: v for k, v in tmp_pred.items()},
                **{"corr_" + k: host(s[k]) for k in ("pos", "vel", "rho", "p")})
            # ---- whole steps from the unperturbed (hydrostatic) state
            d, s, w, tmp = H.alloc(st, cuda)
            H.step(d, s, w, tmp, 1)
            H.sync()
            one = {k: host(d[k]).copy() for k in ("pos", "vel", "rho", "p")}
            H.step(d, s, w, tmp, 4)
            H.sync()
            np.savez_compressed(
                os.path.join(outdir, f"ref_run_{name}.npz"), **common,
                in_pos=st["pos"], in_vel=st["vel"], in_rho=st["rho"], in_p=st["p"], in_type=st["type"],
                **{"step1_" + k: v for k, v in one.items()},
                **{"step5_" + k: host(d[k]) for k in ("pos", "vel", "rho", "p")})
        print(f"{name}: n={n} cells={P.num_cells}", flush=True)


def digest(a) -> str:
    import hashlib
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


REF_RUN_STEPS = 200


def full_size(outdir=HERE):
    import json
    import torch
    from tmp_sph_gb300 import cases
    from oracle import oracle as O
    from oracle.ref_harness import RefHarness
    cuda = torch.device("cuda:0")
    host = lambda t: t.detach().cpu().numpy()
    H = RefHarness()
    # ---- the reference's cell list on the full 4,963,548-particle state
    st, p = cases.build("large", physics="config")
    P = O.params_like(p)
    P.eos = 0
    n = len(st["rho"])
    H.set_params(P, n)
    d, s, w, tmp = H.alloc(st, cuda)
    H.calc_hash(d["pos"], w["hash"], w["index"])
    H.sync()
    hash_unsorted = host(w["hash"]).copy()
    H.sort(w["hash"], w["index"])
    H.reorder(d, s, w["hash"], w["index"], w["cs"], w["ce"])
    H.sync()
    cs = host(w["cs"])[:P.num_cells]
    ce = host(w["ce"])[:P.num_cells]
    occ = cs >= 0
    rec = {"case": "large", "physics": "config", "particles": n, "num_cells": P.num_cells,
           "grid_dim": list(P.grid_dim), "cell_size": float(P.cell_size),
           "occupied_cells": int(occ.sum()),
           "digest": {"in_pos": digest(st["pos"]), "in_vel": digest(st["vel"]),
                      "in_rho": digest(st["rho"]), "in_p": digest(st["p"]),
                      "in_type": digest(st["type"]),
                      "hash_unsorted": digest(hash_unsorted), "hash": digest(host(w["hash"])),
                      "index": digest(host(w["index"])), "cell_start": digest(cs),
                      "cell_end_occupied": digest(ce[occ]),
                      **{"s_" + k: digest(host(s[k])) for k in ("pos", "vel", "rho", "p", "type")}},
           "sample": {"index_first": host(w["index"])[:8].tolist(),
                      "index_last": host(w["index"])[-8:].tolist(),
                      "hash_first": host(w["hash"])[:8].tolist(),
                      "hash_last": host(w["hash"])[-8:].tolist(),
                      "cell_start_first_occupied": int(np.flatnonzero(occ)[0])}}
    with open(os.path.join(outdir, "ref_cells_dam_4963548.json"), "w") as f:
        json.dump(rec, f, indent=1)
    print(f"4,963,548-particle cells: n={n} cells={P.num_cells} occupied={int(occ.sum())}", flush=True)
    del d, s, w, tmp
    torch.cuda.empty_cache()
    # ---- 200 steps of the reference's src step loop on the 133,968-particle dam break
    st, p = cases.build("small", physics="config")
    P = O.params_like(p)
    P.eos = 0
    n = len(st["rho"])
    H.set_params(P, n)
    d, s, w, tmp = H.alloc(st, cuda)
    H.step(d, s, w, tmp, REF_RUN_STEPS)
    H.sync()
    fl = st["type"] == 1
    out = {k: host(d[k])[fl] for k in ("pos", "vel", "rho", "p")}
    np.savez_compressed(os.path.join(outdir, "ref_run_dam_133968.npz"), steps=REF_RUN_STEPS,
                        in_pos_digest=digest(st["pos"]), particles=n,
                        **{"step_" + k: v for k, v in out.items()})
    print(f"133,968-particle run: n={n} steps={REF_RUN_STEPS} finite={np.isfinite(out['vel']).all()}",
          flush=True)


if __name__ == "__main__":
    args = [a for a in sys.argv[1:] if not a.startswith("--")]
    if "--full-size" in sys.argv:
        full_size(args[0] if args else HERE)
    else:
        main(args[0] if args else HERE)
