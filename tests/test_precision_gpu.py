"""GPU tests of the resident solver's three precisions (SPH_OPT_PRECISION).

* FP64 is the accuracy reference: it must agree with the oracle's FP64 restatement of the
  reference step loop to FP64 rounding growth.
* FP32 and the mixed precisions are measured against the FP64 run of the same solver; the bar
  is 1e-3 relative L2 on the flow fields after 1000 steps.
* The mixed-precision neighbour lists and cell walks visit the same pairs in the same order, so
  they agree bit for bit, as in FP32."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


def run_prec(st, p, nsteps, precision, opts=None, graph=True):
    import torch
    from tmp_sph_gb300 import api, solver as S
    n = len(st["rho"])
    s = torch.cuda.Stream()
    with S.Solver(p, n, precision=precision) as sol:
        sol.set_option(api.SPH_OPT_USE_GRAPH, int(graph))
        for k, v in (opts or {}).items():
            sol.set_option(k, v)
        sol.upload(st["pos"], st["vel"], st["rho"], st["p"], st["type"], stream=s)
        sol.step(nsteps, stream=s)
        out = sol.download(stream=s)
        out["f64"] = sol.download_f64(stream=s)
        out["flags"] = sol.error_flags(stream=s)
        out["rebuilds"] = sol.rebuild_count(stream=s)
    return out


def errors(out, ref, st):
    """Relative L2 errors of the fluid fields; `out` and `ref` in full precision."""
    fl = st["type"] == 1
    n_f = int(fl.sum())
    return {
        "disp": rel_l2(out["pos"][fl] - st["pos"][fl], ref["pos"][fl] - st["pos"][fl]),
        "vel": rel_l2(out["vel"][fl], ref["vel"][fl], floor=1e-3 * np.sqrt(n_f)),
        "drho": rel_l2(out["rho"][fl] - 1000.0, ref["rho"][fl] - 1000.0),
        "p": rel_l2(out["p"][fl], ref["p"][fl]),
    }


@pytest.mark.parametrize("physics", ["reference", "config"])
def test_fp64_matches_fp64_oracle(sphlib, oracle, cuda, report, physics):
    """The FP64 solver against the oracle in FP64 (the reference's arithmetic, double).  The
    oracle forms the constant products rho0 cs h, alpha h cs, delta h cs and eta^2 from the
    float parameters in float, as the reference's kernels do; the FP64 solver forms them in
    double.  Those constants differ by up to ~1e-7 relative and move the fields by ~1e-9, two
    orders below the ~1e-5 of FP32 (measured 1 step: vel 1.6e-9 / 2.9e-9, rho 4e-11)."""
    from tmp_sph_gb300 import cases
    st, p = cases.build("small", physics=physics, dx=0.02, jitter=0.01)
    P = oracle.params_like(p)
    for nsteps in (1, 20):
        out = run_prec(st, p, nsteps, "fp64")
        ref = oracle.run(P, st, nsteps, dtype=np.float64)
        assert out["flags"] == 0
        e = errors(out["f64"], ref, st)
        for k, v in e.items():
            report(f"fp64 vs fp64 oracle {physics} {nsteps} steps {k}", v, 1e-7)
        assert all(v < 1e-7 for v in e.values()), e


def test_fp32_and_mixed_against_fp64(sphlib, cuda, report):
    """1000 steps of the small dam break (27,288 particles): FP32 and mixed precision against
    the FP64 run of the same solver, relative L2 of displacement, velocity, rho - rho0, p
    (measured: FP32 3e-5 / 9e-5 / 4e-4 / 4e-4, mixed 1e-6 / 3e-6 / 1.3e-5 / 1.3e-5 with
    compensated sums)."""
    from tmp_sph_gb300 import cases
    st, p = cases.build("small", physics="config", dx=0.02, jitter=0.01)
    steps = 1000
    ref = run_prec(st, p, steps, "fp64")
    assert ref["flags"] == 0
    res = {}
    for prec in ("fp32", "mixed", "mixed_comp", "mixed_abs"):
        out = run_prec(st, p, steps, prec)
        assert out["flags"] == 0, prec
        res[prec] = errors(out["f64"], ref["f64"], st)
        for k, v in res[prec].items():
            report(f"{prec} vs fp64, small case {steps} steps, {k}", v, 1e-3)
    for prec, e in res.items():
        assert all(v < 1e-3 for v in e.values()), (prec, e)


@pytest.mark.parametrize("precision", ["mixed", "mixed_abs"])
def test_mixed_list_matches_cell_walk(sphlib, cuda, precision):
    """Mixed precision: one-lane list passes and walking passes (cell codes from the walk, or
    FP32 positions) agree bit for bit; an overflowing list falls back to the same walk."""
    from tmp_sph_gb300 import api, cases
    st, p = cases.build("small", physics="config", dx=0.02, jitter=0.01)
    one = {api.SPH_OPT_LANES_PER_PARTICLE: 1}
    a = run_prec(st, p, 5, precision, {**one, api.SPH_OPT_SKIN_PERMILLE: 0})
    b = run_prec(st, p, 5, precision, {**one, api.SPH_OPT_SKIN_PERMILLE: 0,
                                       api.SPH_OPT_NEIGHBOR_LIST: 0})
    c = run_prec(st, p, 5, precision, {**one, api.SPH_OPT_NEIGHBOR_CAP: 8})
    d = run_prec(st, p, 5, precision, one)
    assert a["flags"] == 0 and b["flags"] == 0 and d["flags"] == 0
    assert c["flags"] & api.SPH_FLAG_NEIGHBOR_OVERFLOW
    for k in ("pos", "vel", "rho", "p"):
        assert np.array_equal(a[k], b[k]), k
        assert np.array_equal(c[k], d[k]), k


@pytest.mark.parametrize("precision", ["fp64", "mixed", "mixed_abs"])
def test_graph_replay_bitwise(sphlib, cuda, precision):
    from tmp_sph_gb300 import cases
    from gpu_util import perturbed
    st, p = cases.build("small", physics="config", dx=0.02, jitter=0.01)
    st = perturbed(st, vamp=2.0, ramp=0.0)
    a = run_prec(st, p, 7, precision, graph=True)
    b = run_prec(st, p, 7, precision, graph=False)
    assert a["rebuilds"] >= 2
    for k in ("pos", "vel", "rho", "p", "type"):
        assert np.array_equal(a[k], b[k]), k


def test_precision_change_drops_state(sphlib, cuda):
    """Switching precision reallocates the state: stepping needs a new upload."""
    import torch
    from tmp_sph_gb300 import api, cases, solver as S
    st, p = cases.build("small", physics="config", dx=0.04)
    n = len(st["rho"])
    s = torch.cuda.Stream()
    with S.Solver(p, n) as sol:
        sol.upload(st["pos"], st["vel"], st["rho"], st["p"], st["type"], stream=s)
        sol.set_option(api.SPH_OPT_PRECISION, api.SPH_PREC_MIXED)
        assert api.lib().sph_step(sol.handle, 1, None) == api.SPH_ERR_STATE
        sol.upload(st["pos"], st["vel"], st["rho"], st["p"], st["type"], stream=s)
        sol.step(2, stream=s)
        out = sol.download(stream=s)
        assert sol.error_flags(stream=s) == 0
    assert np.isfinite(out["pos"]).all()
