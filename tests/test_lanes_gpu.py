"""GPU tests of the lane-group list pass 1 (SPH_OPT_LANES_PER_PARTICLE = SPH_OPT_PASS1_LANES):
G lanes share one particle's neighbour list and reduce their partial sums with shuffles.  Every G reads the list the one-lane build writes; the sums associate
differently, so the results match the oracle and the one-lane kernels to FP32 rounding; for a
fixed G they are deterministic and independent of the block size, of graph replay, and of
batching."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import rel_l2
from test_solver_gpu import field_errors

pytestmark = pytest.mark.gpu

LANES = [2, 4, 8, 16]


def run(st, p, nsteps, lanes, precision="fp32", opts=None, graph=True):
    import torch
    from tmp_sph_gb300 import api, solver as S
    s = torch.cuda.Stream()
    with S.Solver(p, len(st["rho"]), precision=precision) as sol:
        sol.set_option(api.SPH_OPT_USE_GRAPH, int(graph))
        sol.set_option(api.SPH_OPT_LANES_PER_PARTICLE, lanes)
        for k, v in (opts or {}).items():
            sol.set_option(k, v)
        sol.upload(st["pos"], st["vel"], st["rho"], st["p"], st["type"], stream=s)
        sol.step(nsteps, stream=s)
        out = sol.download(stream=s)
        out["flags"] = sol.error_flags(stream=s)
        out["rebuilds"] = sol.rebuild_count(stream=s)
    return out


def small(perturb=False):
    from tmp_sph_gb300 import cases
    from gpu_util import perturbed
    st, p = cases.build("small", physics="config", dx=0.02, jitter=0.01)
    if perturb:
        st = perturbed(st, vamp=2.0, ramp=0.0)
    return st, p


@pytest.mark.parametrize("lanes", LANES)
def test_lanes_match_oracle(sphlib, oracle, cuda, report, lanes):
    st, p = small()
    P = oracle.params_like(p)
    for nsteps, tol, tol_disp in ((1, 2e-5, 5e-4), (20, 2e-4, 2e-4)):
        out = run(st, p, nsteps, lanes)
        ref = oracle.run(P, st, nsteps)
        assert out["flags"] == 0
        e = field_errors(out, ref, st)
        for k, v in e.items():
            report(f"lanes {lanes}, {nsteps} steps {k}", v, tol_disp if k == "disp" else tol)
        assert e["disp"] < tol_disp and all(v < tol for k, v in e.items() if k != "disp"), e
        wl = st["type"] != 1
        assert np.array_equal(out["pos"][wl], st["pos"][wl])


@pytest.mark.parametrize("lanes", [4, 8])
def test_lanes_close_to_one_lane(sphlib, cuda, report, lanes):
    """Fast flow (list rebuilds along the way): the lane groups follow the one-lane kernels to
    FP32 rounding, with the same rebuild schedule."""
    st, p = small(perturb=True)
    a = run(st, p, 10, 1)
    b = run(st, p, 10, lanes)
    fl = st["type"] == 1
    e = rel_l2(b["vel"][fl], a["vel"][fl], floor=1e-3 * np.sqrt(fl.sum()))
    report(f"lanes {lanes} vs 1, 10 fast steps, vel", e, 1e-5)
    assert e < 1e-5
    assert a["rebuilds"] == b["rebuilds"] and a["rebuilds"] >= 2
    assert a["flags"] == 0 and b["flags"] == 0


def test_lanes_switch(sphlib, cuda, report):
    """Lane groups read interleaved list windows: turning groups on or off rebuilds the lists at
    the next half step; changing G while groups stay on keeps them (the rebuilds follow a run
    without that change).  The run continues either way."""
    import torch
    from tmp_sph_gb300 import api, solver as S
    st, p = small()
    s = torch.cuda.Stream()
    # (option, G, whether the list windows change)
    segments = ((None, 0, False), (api.SPH_OPT_PASS1_LANES, 4, True),
                (api.SPH_OPT_PASS1_LANES, 2, False), (api.SPH_OPT_LANES_PER_PARTICLE, 1, True),
                (api.SPH_OPT_PASS1_LANES, 0, True))
    counts = {}
    for keep_g in (False, True):
        with S.Solver(p, len(st["rho"])) as sol:
            # cells of the list cutoff, where the FP32 default is two lanes
            sol.set_option(api.SPH_OPT_CELL_DIVISIONS, 1)
            sol.set_option(api.SPH_OPT_LANES_PER_PARTICLE, 1)
            sol.upload(st["pos"], st["vel"], st["rho"], st["p"], st["type"], stream=s)
            counts[keep_g] = []
            for opt, g, windows in segments:
                before = sol.rebuild_count(stream=s)
                # the run with keep_g skips the change of G that keeps the windows
                if opt is not None and not (keep_g and not windows):
                    sol.set_option(opt, g)
                sol.step(1, stream=s)
                if windows:
                    assert sol.rebuild_count(stream=s) > before, (opt, g)
                sol.step(3, stream=s)
                counts[keep_g].append(sol.rebuild_count(stream=s))
            if not keep_g:
                assert sol.get_option(api.SPH_OPT_PASS1_LANES) == 2  # the FP32 default
                out = sol.download(stream=s)
            assert sol.error_flags(stream=s) == 0
    assert counts[False] == counts[True], counts
    ref = run(st, p, 20, 1)
    fl = st["type"] == 1
    e = rel_l2(out["vel"][fl], ref["vel"][fl], floor=1e-3 * np.sqrt(fl.sum()))
    report("lane groups for steps 5-12 and 17-20 vs one lane, vel", e, 1e-5)
    assert e < 1e-5


def test_lanes_defaults(sphlib, cuda):
    """Pass 1 takes two lanes per particle in FP32 on cells of the list cutoff while the lists
    have a skin; one on the default FP32 cells of a third of the cutoff, without a skin and in
    the other precisions."""
    from tmp_sph_gb300 import api, solver as S
    st, p = small()
    for prec, want in (("fp32", 2), ("mixed", 1), ("mixed_comp", 1), ("fp64", 1)):
        with S.Solver(p, len(st["rho"]), precision=prec) as sol:
            assert sol.get_option(api.SPH_OPT_PASS1_LANES) == 1, prec
            sol.set_option(api.SPH_OPT_CELL_DIVISIONS, 1)
            assert sol.get_option(api.SPH_OPT_PASS1_LANES) == want, prec
            sol.set_option(api.SPH_OPT_SKIN_PERMILLE, 0)
            assert sol.get_option(api.SPH_OPT_PASS1_LANES) == 1, prec


@pytest.mark.parametrize("precision,tol", [("mixed", 1e-4), ("mixed_comp", 1e-4), ("fp64", 1e-7)])
def test_lanes_other_precisions(sphlib, oracle, cuda, report, precision, tol):
    """Against the oracle in FP64: the FP64 solver to its constants' rounding (as with one
    lane), mixed precision to its FP32 pair arithmetic."""
    from test_precision_gpu import errors, run_prec
    from tmp_sph_gb300 import api
    st, p = small()
    out = run_prec(st, p, 5, precision, opts={api.SPH_OPT_LANES_PER_PARTICLE: 8})
    ref = oracle.run(oracle.params_like(p), st, 5, dtype=np.float64)
    e = errors(out["f64"], ref, st)
    for k, v in e.items():
        report(f"lanes 8 {precision} vs fp64 oracle, 5 steps {k}", v, tol)
    assert out["flags"] == 0
    assert all(v < tol for v in e.values()), e


def test_lanes_deterministic_across_shapes_and_graphs(sphlib, cuda):
    from tmp_sph_gb300 import api
    st, p = small(perturb=True)
    ref = run(st, p, 6, 8)
    for opts, graph in (({api.SPH_OPT_BLOCK_THREADS: 64}, True),
                        ({api.SPH_OPT_BLOCK_THREADS: 256}, True),
                        ({}, False),
                        ({api.SPH_OPT_CONDITIONAL_GRAPH: 0}, True)):
        out = run(st, p, 6, 8, opts=opts, graph=graph)
        for k in ("pos", "vel", "rho", "p"):
            assert np.array_equal(out[k], ref[k]), (opts, graph, k)


def test_lanes_overflow_walks(sphlib, cuda, report):
    """With a 16-slot list every fluid particle overflows and its group walks the cells."""
    from tmp_sph_gb300 import api
    st, p = small()
    for skin in (0, 100):
        a = run(st, p, 3, 8, opts={api.SPH_OPT_SKIN_PERMILLE: skin, api.SPH_OPT_NEIGHBOR_CAP: 16})
        b = run(st, p, 3, 8, opts={api.SPH_OPT_SKIN_PERMILLE: skin})
        assert a["flags"] & api.SPH_FLAG_NEIGHBOR_OVERFLOW and b["flags"] == 0
        fl = st["type"] == 1
        e = rel_l2(a["vel"][fl], b["vel"][fl], floor=1e-3 * np.sqrt(fl.sum()))
        report(f"lanes 8 overflow walk vs list, skin {skin}, vel", e, 1e-5)
        assert e < 1e-5


def test_lanes_batch_equals_solo(sphlib, cuda):
    import torch
    from tmp_sph_gb300 import api, cases, solver as S
    states, p = cases.batch(2, dx=0.02, seed=9)
    n = sum(len(st["rho"]) for st in states)
    s = torch.cuda.Stream()
    with S.Solver(p, n) as sol:
        sol.set_option(api.SPH_OPT_SKIN_PERMILLE, 0)
        sol.set_option(api.SPH_OPT_LANES_PER_PARTICLE, 8)
        off = sol.upload_instances(states, stream=s)
        sol.step(3, stream=s)
        out = sol.download(stream=s)
        assert sol.error_flags(stream=s) == 0
    for b, st in enumerate(states):
        ref = run(st, p, 3, 8, opts={api.SPH_OPT_SKIN_PERMILLE: 0})
        sl = slice(int(off[b]), int(off[b + 1]))
        for k in ("pos", "vel", "rho", "p"):
            assert np.array_equal(out[k][sl], ref[k]), (b, k)


@pytest.mark.parametrize("cap", [32, 48, 64])
def test_interleaved_windows_at_small_capacities(sphlib, oracle, cuda, report, cap):
    """Lists of 32-64 slots: counts end in every position of a window of eight, reach the
    capacity exactly, or pass it (those particles walk their cells).  Pass 1 with two and
    four lanes over the interleaved windows follows the one-lane run to FP32 rounding and the
    oracle within the step tolerance."""
    from tmp_sph_gb300 import api
    st, p = small()
    opts = {api.SPH_OPT_NEIGHBOR_CAP: cap}
    one = run(st, p, 4, 1, opts=opts)
    ref = oracle.run(oracle.params_like(p), st, 4)
    fl = st["type"] == 1
    for g in (2, 4):
        out = run(st, p, 4, 1, opts={**opts, api.SPH_OPT_PASS1_LANES: g})
        assert (out["flags"] & ~api.SPH_FLAG_NEIGHBOR_OVERFLOW) == 0
        e = rel_l2(out["vel"][fl], one["vel"][fl], floor=1e-3 * np.sqrt(fl.sum()))
        report(f"cap {cap}, pass-1 lanes {g} vs one lane, 4 steps, vel", e, 1e-5)
        assert e < 1e-5
        errs = field_errors(out, ref, st)
        assert all(v < 2e-4 for v in errs.values()), (g, errs)


def test_lanes_option_checked(sphlib):
    from tmp_sph_gb300 import api, cases, solver as S
    st, p = small()
    with S.Solver(p, len(st["rho"])) as sol:
        for bad in (3, 32, -1):
            with pytest.raises(api.SphError):
                sol.set_option(api.SPH_OPT_LANES_PER_PARTICLE, bad)
        for good in (0, 1, 2, 4, 8, 16):
            sol.set_option(api.SPH_OPT_LANES_PER_PARTICLE, good)
        with pytest.raises(api.SphError):
            sol.set_option(api.SPH_OPT_PASS1_LANES, 5)
        sol.set_option(api.SPH_OPT_PASS1_LANES, 4)
        assert sol.get_option(api.SPH_OPT_PASS1_LANES) == 4
        assert sol.get_option(api.SPH_OPT_LANES_PER_PARTICLE) == 4
        # the retired options (pair mode 11, pass-2 lane groups 15) are refused
        for retired in (11, 15):
            with pytest.raises(api.SphError):
                sol.set_option(retired, 1)
