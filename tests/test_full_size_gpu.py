"""Parity at the benchmark configurations themselves (not only at the small fixture sizes).

* the 4,963,548-particle dam break (dx 2.5 mm, seeded jitter): the drop-in calcHash ->
  sortParticles -> reorder chain gives the reference's own output bit for bit (SHA-256
  digests of every array its kernels produced on the same input, tests/golden/
  ref_cells_dam_4963548.json); one resident FP32 step matches the oracle's step; the project's
  radix sort equals a stable argsort on the real cell keys of this state.
* the batched workload (64 dam breaks, 48.9M particles): the radix sort equals a
  stable argsort on the stacked instance keys (25 bits).
* the 133,968-particle dam break (dx 1 cm, h = 1.3 dx, the reference's linear EOS): 200 resident
  steps against 200 steps of the reference's own src step loop (tests/golden/
  ref_run_dam_133968.npz).
* the 765,828-particle dam break (dx 5 mm): mixed precision within 1e-3 of the FP64 solver after
  1000 steps.
"""
from __future__ import annotations

import hashlib
import json
import os

import numpy as np
import pytest

from conftest import rel_l2
from gpu_util import dev, host

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def digest(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.fixture(scope="module")
def large():
    from tmp_sph_gb300 import cases
    return cases.build("large", physics="config")


def test_dam_4963548_cells_match_reference(sphlib, cuda, large):
    """calcHash -> sortParticles -> reorder (src/lib/mesh.cu:26-159) through the drop-in C ABI
    at the full 4,963,548-particle size: hash, index, cellStart, cellEnd of the occupied cells and
    every gathered array identical to the reference's."""
    import torch
    from tmp_sph_gb300 import api, solver as S
    with open(os.path.join(GOLD, "ref_cells_dam_4963548.json")) as f:
        ref = json.load(f)
    st, p = large
    p.eos = api.SPH_EOS_LINEAR
    n = len(st["rho"])
    assert n == ref["particles"] and p.num_cells == ref["num_cells"]
    assert digest(st["pos"]) == ref["digest"]["in_pos"], "generator output differs from the fixture's input"
    pos = dev(st["pos"], cuda)
    h = torch.empty(n, dtype=torch.int32, device=cuda)
    idx = torch.empty(n, dtype=torch.int32, device=cuda)
    S.calc_hash(p, pos, h, idx, n)
    assert digest(host(h)) == ref["digest"]["hash_unsorted"]
    S.sort_particles(h, idx, n)
    out = {k: torch.empty_like(dev(st[k], cuda)) for k in ("pos", "vel", "rho", "p", "type")}
    cs = torch.empty(p.num_cells, dtype=torch.int32, device=cuda)
    ce = torch.full((p.num_cells,), -7, dtype=torch.int32, device=cuda)
    S.reorder(p, pos, dev(st["vel"], cuda), dev(st["rho"], cuda), dev(st["p"], cuda),
              dev(st["type"], cuda), None, out["pos"], out["vel"], out["rho"], out["p"],
              out["type"], None, h, idx, cs, ce, n)
    hh, ii, cc, ee = host(h), host(idx), host(cs), host(ce)
    assert hh[:8].tolist() == ref["sample"]["hash_first"]
    assert ii[:8].tolist() == ref["sample"]["index_first"]
    assert ii[-8:].tolist() == ref["sample"]["index_last"]
    assert digest(hh) == ref["digest"]["hash"]
    assert digest(ii) == ref["digest"]["index"]
    assert digest(cc) == ref["digest"]["cell_start"]
    occ = cc >= 0
    assert int(occ.sum()) == ref["occupied_cells"]
    assert digest(ee[occ]) == ref["digest"]["cell_end_occupied"]
    for k in out:
        assert digest(host(out[k])) == ref["digest"]["s_" + k], k


def test_dam_4963548_keys_radix_sort_matches_stable_argsort(sphlib, cuda, large):
    """The project's radix sort on the 4,963,548 real cell keys of the 4.96M dam break (22-bit
    range), against numpy's stable argsort, with the key width the solver uses and with 32 bits."""
    import torch
    from tmp_sph_gb300 import solver as S
    st, p = large
    n = len(st["rho"])
    pos = dev(st["pos"], cuda)
    h = torch.empty(n, dtype=torch.int32, device=cuda)
    idx = torch.empty(n, dtype=torch.int32, device=cuda)
    S.calc_hash(p, pos, h, idx, n)
    keys = host(h)
    assert keys.min() >= 0 and keys.max() < p.num_cells < 2 ** 22
    order = np.argsort(keys, kind="stable")
    vals = np.random.default_rng(3).permutation(n).astype(np.int32)
    for kb in (22, 32):
        hk, vk = dev(keys, cuda), dev(vals, cuda)
        S.sort_particles(hk, vk, n, key_bits=kb)
        assert np.array_equal(host(hk), keys[order]), kb
        assert np.array_equal(host(vk), vals[order]), kb


def test_batch_keys_radix_sort_matches_stable_argsort(sphlib, cuda):
    """The batched workload's keys: 64 dam breaks of uneven size (48.9M particles), each
    instance's cells stacked after the previous instance's (25-bit keys), sorted by the radix
    sort and by numpy's stable argsort."""
    import torch
    from tmp_sph_gb300 import cases, solver as S
    states, p = cases.batch(64)
    gmin = np.asarray(p.grid_min, np.float32)
    cell = np.float32(p.cell_size)
    dims = np.asarray(p.grid_dim, np.int64)
    per_inst = int(dims[0] * dims[1] * (dims[2] + 1))
    parts = []
    for b, st in enumerate(states):
        c = np.floor((st["pos"] - gmin) / cell).astype(np.int64)
        c = np.clip(c, 0, dims - 1)
        parts.append(b * per_inst + (c[:, 2] * dims[1] + c[:, 1]) * dims[0] + c[:, 0])
    keys = np.concatenate(parts)
    n = len(keys)
    bits = int(keys.max()).bit_length()
    assert n > 40_000_000 and bits == 25
    keys = keys.astype(np.int32)
    order = np.argsort(keys, kind="stable")
    vals = np.arange(n, dtype=np.int32)
    hk, vk = dev(keys, cuda), dev(vals, cuda)
    S.sort_particles(hk, vk, n, key_bits=bits)
    torch.cuda.synchronize()
    assert np.array_equal(host(vk), order.astype(np.int32))
    assert np.array_equal(host(hk), keys[order])


def test_dam_4963548_one_step_matches_oracle(sphlib, oracle, cuda, report, large):
    """One resident FP32 step of the 4,963,548-particle dam break against one step of the
    oracle (the C restatement of src/sph/sph_run.cu:285-336) on the same input: relative L2 of
    the fluid velocity and density perturbation below 1e-4 (float rounding of sums taken in
    another order; the cell lists of both are bit-exact, above).  One step from rest moves a
    particle by about g dt^2 ~ 1e-8 m, below the spacing of float positions near 0.5 m
    (6e-8 m), so positions are compared in units of that spacing: at most 8 apart (the GPU
    fuses the x + dt/2 v multiply-add, the oracle rounds twice)."""
    import torch
    from tmp_sph_gb300 import solver as S
    st, p = large
    n = len(st["rho"])
    s = torch.cuda.Stream()
    with S.Solver(p, n) as sol:
        sol.upload(st["pos"], st["vel"], st["rho"], st["p"], st["type"], stream=s)
        sol.step(1, stream=s)
        out = sol.download(stream=s)
        assert sol.error_flags(stream=s) == 0
    ref = oracle.run(oracle.params_like(p), st, 1)
    fl = st["type"] == 1
    spacing = np.spacing(np.abs(ref["pos"][fl]).astype(np.float32)).astype(np.float64)
    ulps = float(np.max(np.abs(out["pos"][fl].astype(np.float64) - ref["pos"][fl]) / spacing))
    e_v = rel_l2(out["vel"][fl], ref["vel"][fl])
    e_r = rel_l2(out["rho"][fl] - 1000.0, ref["rho"][fl] - 1000.0)
    report("dam4963548_step1_pos_max_ulps", ulps, 8)
    report("dam4963548_step1_vel", e_v, 1e-4)
    report("dam4963548_step1_drho", e_r, 1e-4)
    assert ulps <= 8 and e_v < 1e-4 and e_r < 1e-4, (ulps, e_v, e_r)


REF_RUN_TOL = 2e-4  # measured 1.2e-5 / 6.0e-6 / 4.0e-5 / 4.0e-5 on a GB300


def test_dam_133968_200_steps_match_reference(sphlib, cuda, report):
    """200 resident FP32 steps of the 133,968-particle dam break against 200 steps of the
    reference's own src step loop (its kernels compiled from its sources, run on a GB300:
    tests/golden/ref_run_dam_133968.npz), same input and constants (h = 1.3 dx, c0 = 24.26 m/s,
    delta 0.1, alpha 0.02, dt = 0.25 h / c0, linear EOS). Relative L2 over the fluid of
    displacement, velocity, rho - rho0 and p within REF_RUN_TOL (the sums run in another order, and
    the differences grow with the flow)."""
    import torch
    from tmp_sph_gb300 import api, cases, solver as S
    d = np.load(os.path.join(GOLD, "ref_run_dam_133968.npz"))
    st, p = cases.build("small", physics="config")
    p.eos = api.SPH_EOS_LINEAR
    n = len(st["rho"])
    assert n == int(d["particles"]) == 133968
    assert digest(st["pos"]) == str(d["in_pos_digest"])
    steps = int(d["steps"])
    s = torch.cuda.Stream()
    with S.Solver(p, n) as sol:
        sol.upload(st["pos"], st["vel"], st["rho"], st["p"], st["type"], stream=s)
        sol.step(steps, stream=s)
        out = sol.download(stream=s)
        assert sol.error_flags(stream=s) == 0
    fl = st["type"] == 1
    x0 = st["pos"][fl]
    errs = {"disp": rel_l2(out["pos"][fl] - x0, d["step_pos"] - x0),
            "vel": rel_l2(out["vel"][fl], d["step_vel"]),
            "drho": rel_l2(out["rho"][fl] - 1000.0, d["step_rho"] - 1000.0),
            "p": rel_l2(out["p"][fl], d["step_p"])}
    for k, v in errs.items():
        report(f"dam133968_{steps}steps_{k}", v, REF_RUN_TOL)
    assert all(v < REF_RUN_TOL for v in errs.values()), errs


def test_dam_765828_mixed_within_1e3_of_fp64_after_1000_steps(sphlib, cuda, report):
    """The precision claim at its configuration: 765,828 particles, 1000 steps; mixed precision
    (FP32 neighbour sums on cell-relative positions, FP64 positions and rho - rho0) and its
    variant on FP32 positions (mixed_abs) against the FP64 solver, relative L2 over the fluid of
    displacement, velocity, rho - rho0 and p below 1e-3."""
    import torch
    from tmp_sph_gb300 import cases, solver as S
    st, p = cases.build("precision", physics="config")
    n = len(st["rho"])
    s = torch.cuda.Stream()
    res = {}
    for prec in ("fp64", "mixed", "mixed_abs"):
        with S.Solver(p, n, precision=prec) as sol:
            sol.upload(st["pos"], st["vel"], st["rho"], st["p"], st["type"], stream=s)
            sol.step(1000, stream=s)
            res[prec] = sol.download_f64(stream=s)
            assert sol.error_flags(stream=s) == 0
    fl = st["type"] == 1
    x0 = st["pos"][fl].astype(np.float64)
    b = res["fp64"]
    for prec in ("mixed", "mixed_abs"):
        a = res[prec]
        errs = {"disp": rel_l2(a["pos"][fl] - x0, b["pos"][fl] - x0),
                "vel": rel_l2(a["vel"][fl], b["vel"][fl]),
                "drho": rel_l2(a["rho"][fl] - 1000.0, b["rho"][fl] - 1000.0),
                "p": rel_l2(a["p"][fl], b["p"][fl])}
        for k, v in errs.items():
            report(f"dam765828_{prec}_vs_fp64_1000_{k}", v, 1e-3)
        assert all(v < 1e-3 for v in errs.values()), (prec, errs)
