"""GPU tests of batched instances (sph_upload_instances): several independent dam breaks
advanced by the same launches.  The instances are stacked in one grid with empty cell layers
between them, so every instance sees exactly the neighbours, in exactly the order, it would see
alone when its lists are rebuilt on the same schedule.  With per-instance decisions
(SPH_OPT_INSTANCE_DECISIONS 1) each instance keeps its own displacement box and skin and
rebuilds exactly when it would alone, so each instance of a batched run equals its solo run bit
for bit, with the skin on or off.  With one decision for the batch (the default) the batch
rebuilds when any instance needs it, so summation orders — not the pairs — can differ from a
solo run: agreement to FP32 rounding, bit for bit without a skin."""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def solo(st, p, nsteps, precision, skin=100):
    import torch
    from tmp_sph_gb300 import api, solver as S
    s = torch.cuda.Stream()
    with S.Solver(p, len(st["rho"]), precision=precision) as sol:
        sol.set_option(api.SPH_OPT_SKIN_PERMILLE, skin)
        sol.upload(st["pos"], st["vel"], st["rho"], st["p"], st["type"], stream=s)
        sol.step(nsteps, stream=s)
        out = sol.download(stream=s)
        out["flags"] = sol.error_flags(stream=s)
        out["rebuilds"] = sol.rebuild_count(stream=s)
        _, out["stats"] = sol.probe(stream=s)
    return out


@pytest.mark.parametrize("precision,skin,own", [("fp32", 0, 1), ("mixed", 0, 1), ("fp32", 100, 1),
                                                ("mixed", 100, 1), ("mixed_abs", 100, 1),
                                                ("fp32", 100, 0)])
def test_batched_instances_equal_solo_runs(sphlib, cuda, report, precision, skin, own):
    import torch
    from tmp_sph_gb300 import api, cases, solver as S
    from gpu_util import perturbed
    from conftest import rel_l2
    states, p = cases.batch(3, dx=0.02, seed=11)
    states[1] = perturbed(states[1], vamp=1.0, ramp=0.0)  # one instance with fast flow
    n = sum(len(st["rho"]) for st in states)
    steps = 12
    s = torch.cuda.Stream()
    with S.Solver(p, n, precision=precision) as sol:
        sol.set_option(api.SPH_OPT_SKIN_PERMILLE, skin)
        sol.set_option(api.SPH_OPT_INSTANCE_DECISIONS, own)
        off = sol.upload_instances(states, stream=s)
        ni = ctypes.c_int(0)
        api.lib().sph_instances(sol.handle, ctypes.byref(ni))
        assert ni.value == 3
        sol.step(steps, stream=s)
        out = sol.download(stream=s)
        flags = sol.error_flags(stream=s)
        _, stats = sol.probe(stream=s)
        rebuilds = sol.rebuild_count(stream=s)
        per_inst = sol.instance_rebuild_counts(3, stream=s)
    assert flags == 0
    assert rebuilds >= 2
    report(f"batched {precision} skin {skin} rebuilds", rebuilds)
    fluid = 0
    solo_rebuilds = []
    for b, st in enumerate(states):
        ref = solo(st, p, steps, precision, skin)
        assert ref["flags"] == 0
        solo_rebuilds.append(ref["rebuilds"])
        sl = slice(int(off[b]), int(off[b + 1]))
        fl = st["type"] == 1
        if skin == 0 or own:
            for k in ("pos", "vel", "rho", "p", "type"):
                assert np.array_equal(out[k][sl], ref[k]), (b, k)
        else:
            e = rel_l2(out["vel"][sl][fl], ref["vel"][fl], floor=1e-3 * np.sqrt(fl.sum()))
            report(f"batched fp32 skin instance {b} vel", e, 1e-4)
            assert e < 1e-4
            assert np.array_equal(out["type"][sl], ref["type"])
        fluid += ref["stats"]["fluid"]
    assert stats["fluid"] == fluid
    if own:
        # each instance rebuilt exactly when it did alone; the batch when any did
        assert per_inst.tolist() == solo_rebuilds
        assert max(solo_rebuilds) <= rebuilds <= sum(solo_rebuilds)
        if skin:
            assert len(set(solo_rebuilds)) > 1, solo_rebuilds  # the instances' schedules differ
    else:
        assert per_inst.tolist() == [rebuilds] * 3


def test_batched_then_single_upload(sphlib, cuda):
    """sph_upload after a batched upload returns the context to one simulation."""
    import torch
    from tmp_sph_gb300 import api, cases, solver as S
    states, p = cases.batch(2, dx=0.02, seed=3)
    n = sum(len(st["rho"]) for st in states)
    s = torch.cuda.Stream()
    with S.Solver(p, n) as sol:
        sol.set_option(api.SPH_OPT_SKIN_PERMILLE, 0)
        sol.upload_instances(states, stream=s)
        sol.step(2, stream=s)
        st = states[0]
        sol.upload(st["pos"], st["vel"], st["rho"], st["p"], st["type"], stream=s)
        ni = ctypes.c_int(0)
        api.lib().sph_instances(sol.handle, ctypes.byref(ni))
        assert ni.value == 1
        sol.step(3, stream=s)
        out = sol.download(stream=s)
        assert sol.error_flags(stream=s) == 0
    ref = solo(st, p, 3, "fp32", skin=0)
    for k in ("pos", "vel", "rho", "p"):
        assert np.array_equal(out[k], ref[k]), k


def test_instance_offsets_are_checked(sphlib, cuda):
    from tmp_sph_gb300 import api, cases, solver as S
    states, p = cases.batch(2, dx=0.04, seed=5)
    cat = {k: np.ascontiguousarray(np.concatenate([s[k] for s in states]),
                                   np.int32 if k == "type" else np.float32)
           for k in ("pos", "vel", "rho", "p", "type")}
    n = len(cat["rho"])
    lib = api.lib()
    with S.Solver(p, n) as sol:
        def up(off, n_inst, nn=n):
            o = np.ascontiguousarray(off, np.int32)
            return lib.sph_upload_instances(sol.handle, cat["pos"].ctypes.data,
                                            cat["vel"].ctypes.data, cat["rho"].ctypes.data,
                                            cat["p"].ctypes.data, cat["type"].ctypes.data,
                                            o.ctypes.data, n_inst, nn, 1, None)
        n0 = len(states[0]["rho"])
        assert up([0, n0, n - 1], 2) == api.SPH_ERR_ARG       # last offset != n
        assert up([1, n0, n], 2) == api.SPH_ERR_ARG           # first offset != 0
        assert up([0, n, n0], 2) == api.SPH_ERR_ARG           # decreasing
        assert up([0, n0, n], 0) == api.SPH_ERR_ARG           # no instance
        assert up([0] * 4098, api.SPH_MAX_INSTANCES + 1, 0) == api.SPH_ERR_ARG
        assert up([0, n0, n], 2) == api.SPH_OK
