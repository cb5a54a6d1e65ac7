"""GPU tests of the cell-size option (SPH_OPT_CELL_DIVISIONS): the resident grid's cells are
a half or a third of the list cutoff and the cell walks cover 125 or 343 cells.  The walk
finds the same pairs in another order, so the fields follow the oracle to FP32 rounding; with
one lane per particle the neighbour-list passes and the passes that walk the cells themselves
still visit the same pairs in the same order (bitwise); batched instances stay apart (the
stacked grid keeps at least as many empty layers between instances as cells are walked on each
side), so each instance of a batch equals its solo run bit for bit with the lists rebuilt every
half step."""
from __future__ import annotations

import numpy as np
import pytest

from test_solver_gpu import field_errors

pytestmark = pytest.mark.gpu


def run(st, p, nsteps, precision="fp32", opts=None):
    import torch
    from tmp_sph_gb300 import api, solver as S
    s = torch.cuda.Stream()
    with S.Solver(p, len(st["rho"]), precision=precision) as sol:
        for k, v in (opts or {}).items():
            sol.set_option(k, v)
        sol.upload(st["pos"], st["vel"], st["rho"], st["p"], st["type"], stream=s)
        sol.step(nsteps, stream=s)
        out = sol.download(stream=s)
        out["flags"] = sol.error_flags(stream=s)
        out["rebuilds"] = sol.rebuild_count(stream=s)
        if api.SPH_OPT_CELL_DIVISIONS in (opts or {}):
            assert sol.get_option(api.SPH_OPT_CELL_DIVISIONS) == opts[api.SPH_OPT_CELL_DIVISIONS]
    return out


@pytest.mark.parametrize("div", [2, 3])
@pytest.mark.parametrize("precision", ["fp32", "mixed", "mixed_abs"])
def test_divisions_match_oracle(sphlib, oracle, cuda, report, div, precision):
    from tmp_sph_gb300 import api, cases
    from gpu_util import perturbed
    st, p = cases.build("small", physics="config", dx=0.02, jitter=0.01)
    st = perturbed(st, vamp=1.0, ramp=0.0)  # moving particles: several list rebuilds
    out = run(st, p, 20, precision, {api.SPH_OPT_CELL_DIVISIONS: div})
    ref = oracle.run(oracle.params_like(p), st, 20)
    assert out["flags"] == 0 and out["rebuilds"] >= 3
    e = field_errors(out, ref, st)
    for k, v in e.items():
        report(f"cells 1/{div} {precision} 20 steps vs oracle {k}", v, 2e-4)
    assert all(v < 2e-4 for v in e.values()), e


@pytest.mark.parametrize("div", [2, 3])
def test_divisions_list_equals_walk(sphlib, cuda, div):
    """One lane per particle: the list passes and the walking passes agree bit for bit."""
    from tmp_sph_gb300 import api, cases
    from gpu_util import perturbed
    st, p = cases.build("small", physics="config", dx=0.02, jitter=0.01)
    st = perturbed(st, vamp=1.0, ramp=0.0)
    base = {api.SPH_OPT_CELL_DIVISIONS: div, api.SPH_OPT_LANES_PER_PARTICLE: 1,
            api.SPH_OPT_SKIN_PERMILLE: 0}
    a = run(st, p, 6, opts={**base, api.SPH_OPT_NEIGHBOR_LIST: 1})
    b = run(st, p, 6, opts={**base, api.SPH_OPT_NEIGHBOR_LIST: 0})
    for k in ("pos", "vel", "rho", "p"):
        assert np.array_equal(a[k], b[k]), k


@pytest.mark.parametrize("div", [2, 3])
@pytest.mark.parametrize("precision", ["fp32", "mixed", "mixed_abs"])
def test_divisions_batch_equals_solo(sphlib, cuda, div, precision):
    """Mixed precision anchors a particle's offsets at a cell whose coordinates are multiples of
    the reach; the instances are stacked every multiple of the reach, so an instance's anchors,
    offsets and sums are those of its solo run."""
    import torch
    from tmp_sph_gb300 import api, cases, solver as S
    states, p = cases.batch(3, dx=0.02, seed=5)
    n = sum(len(st["rho"]) for st in states)
    opts = {api.SPH_OPT_CELL_DIVISIONS: div, api.SPH_OPT_SKIN_PERMILLE: 0}
    s = torch.cuda.Stream()
    with S.Solver(p, n, precision=precision) as sol:
        for k, v in opts.items():
            sol.set_option(k, v)
        off = sol.upload_instances(states, stream=s)
        sol.step(5, stream=s)
        out = sol.download(stream=s)
        assert sol.error_flags(stream=s) == 0
    for b, st in enumerate(states):
        ref = run(st, p, 5, precision, opts=opts)
        sl = slice(int(off[b]), int(off[b + 1]))
        for k in ("pos", "vel", "rho", "p"):
            assert np.array_equal(out[k][sl], ref[k]), (b, k)


def test_divisions_switch_and_checks(sphlib, cuda):
    """Changing the cell size between steps rebuilds the lists on the new grid and the run
    continues with the same pairs; out-of-range values are refused."""
    import torch
    from tmp_sph_gb300 import api, cases, solver as S
    from conftest import rel_l2
    st, p = cases.build("small", physics="config", dx=0.02, jitter=0.01)
    s = torch.cuda.Stream()
    with S.Solver(p, len(st["rho"])) as sol:
        assert sol.get_option(api.SPH_OPT_CELL_DIVISIONS) == 3  # the FP32 default
        for bad in (4, -1):
            with pytest.raises(api.SphError):
                sol.set_option(api.SPH_OPT_CELL_DIVISIONS, bad)
        sol.set_option(api.SPH_OPT_CELL_DIVISIONS, 1)
        sol.upload(st["pos"], st["vel"], st["rho"], st["p"], st["type"], stream=s)
        sol.step(3, stream=s)
        r0 = sol.rebuild_count(stream=s)
        sol.set_option(api.SPH_OPT_CELL_DIVISIONS, 2)
        sol.step(1, stream=s)
        assert sol.rebuild_count(stream=s) > r0
        sol.step(2, stream=s)
        out = sol.download(stream=s)
        assert sol.error_flags(stream=s) == 0
    ref = run(st, p, 6)
    fl = st["type"] == 1
    e = rel_l2(out["vel"][fl], ref["vel"][fl], floor=1e-3 * np.sqrt(fl.sum()))
    assert e < 1e-5, e


def test_divisions_defaults(sphlib, cuda):
    """Cells of a third of the list cutoff with the FP32 pair arithmetic (FP32 and mixed on
    FP32 positions), of the cutoff in the other precisions; a precision change moves the
    default along unless the caller set the cell size."""
    from tmp_sph_gb300 import api, cases, solver as S
    _, p = cases.build("small", physics="config", dx=0.04)
    for prec, want in (("fp32", 3), ("mixed", 1), ("mixed_comp", 1), ("mixed_abs", 3),
                       ("fp64", 1)):
        with S.Solver(p, 1000, precision=prec) as sol:
            assert sol.get_option(api.SPH_OPT_CELL_DIVISIONS) == want, prec
    with S.Solver(p, 1000) as sol:
        sol.set_option(api.SPH_OPT_CELL_DIVISIONS, 2)
        sol.set_option(api.SPH_OPT_PRECISION, api.PRECISIONS["mixed"])
        assert sol.get_option(api.SPH_OPT_CELL_DIVISIONS) == 2
        sol.set_option(api.SPH_OPT_CELL_DIVISIONS, 0)
        assert sol.get_option(api.SPH_OPT_CELL_DIVISIONS) == 1
