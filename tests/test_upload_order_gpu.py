"""GPU tests of uploads into the current cell order.

After a half step the live set is in the order its cell starts and neighbour lists were built
for.  An upload of the same particles (same count and instances) then goes straight into that
order: slot k takes particle id[k], and the half step's displacement test decides whether the
lists still cover every pair, exactly as it does after a pass-2 update.  So a loop of end-to-end
host calls (sph_step_host: upload, step, download) evaluates the same pairs in the same order as
one resident run and gives the same bits in FP32; moved particles or changed particle kinds
trigger the rebuild the resident path would need."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


def _pinned(st):
    import torch
    return {k: torch.from_numpy(np.ascontiguousarray(st[k])).pin_memory().numpy()
            for k in ("pos", "vel", "rho", "p", "type")}


def _resident(st, p, nsteps, precision="fp32", skin=100):
    import torch
    from tmp_sph_gb300 import api, solver as S
    s = torch.cuda.Stream()
    with S.Solver(p, len(st["rho"]), precision=precision) as sol:
        sol.set_option(api.SPH_OPT_SKIN_PERMILLE, skin)
        sol.upload(st["pos"], st["vel"], st["rho"], st["p"], st["type"], stream=s)
        sol.step(nsteps, stream=s)
        out = sol.download(stream=s)
        out["rebuilds"] = sol.rebuild_count(stream=s)
        out["flags"] = sol.error_flags(stream=s)
    return out


@pytest.mark.parametrize("vamp", [0.3, 2.0])
def test_host_loop_equals_resident_run(sphlib, cuda, report, vamp):
    """12 one-step host calls give the bits of one 12-step resident run, with (±2 m/s) and
    without list rebuilds along the way; the rebuild count keeps counting across the calls
    (a fresh upload would restart it at the forced first rebuild)."""
    import torch
    from tmp_sph_gb300 import api, cases, solver as S
    from gpu_util import perturbed
    st, p = cases.build("small", physics="config", dx=0.02, jitter=0.01)
    st = perturbed(st, vamp=vamp, ramp=0.0)
    steps = 12
    ref = _resident(st, p, steps)
    hst = _pinned(st)
    s = torch.cuda.Stream()
    with S.Solver(p, len(st["rho"])) as sol:
        sol.set_option(api.SPH_OPT_SKIN_PERMILLE, 100)
        for _ in range(steps):
            sol.step_host(hst, 1, stream=s)
        rebuilds = sol.rebuild_count(stream=s)
        flags = sol.error_flags(stream=s)
    assert flags == 0 and ref["flags"] == 0
    for k in ("pos", "vel", "rho", "p"):
        assert np.array_equal(hst[k], ref[k]), k
    report(f"host loop vamp {vamp} rebuilds (resident run)", rebuilds, ref["rebuilds"])
    assert rebuilds == ref["rebuilds"]
    if vamp > 1.0:
        assert rebuilds >= 3


def test_moved_particles_rebuild(sphlib, oracle, cuda, report):
    """An upload that moves particles by more than half the skin rebuilds the lists before the
    next pass; one that moves them less keeps the lists; both match the oracle."""
    import torch
    from tmp_sph_gb300 import api, cases, solver as S
    from test_solver_gpu import field_errors
    st, p = cases.build("small", physics="config", dx=0.02, jitter=0.01)
    skin = 0.1 * 2.0 * p.h  # kh with the Wendland kernel's kappa = 2
    fl = np.nonzero(st["type"] == 1)[0]
    P = oracle.params_like(p)
    s = torch.cuda.Stream()
    with S.Solver(p, len(st["rho"])) as sol:
        sol.set_option(api.SPH_OPT_SKIN_PERMILLE, 100)
        sol.set_option(api.SPH_OPT_ADAPTIVE_SKIN, 0)  # the shifts are measured in this skin
        hst = _pinned(st)
        sol.step_host(hst, 1, stream=s)
        base = sol.rebuild_count(stream=s)
        for shift, expect_rebuild in ((0.2 * skin, False), (0.8 * skin, True)):
            cur = {k: hst[k].copy() for k in hst}
            cur["pos"][fl[::7], 0] += np.float32(shift)
            want = oracle.run(P, cur, 1)
            for k in hst:
                hst[k][...] = cur[k]
            sol.step_host(hst, 1, stream=s)
            n_rb = sol.rebuild_count(stream=s)
            assert (n_rb > base) == expect_rebuild, (shift, base, n_rb)
            base = n_rb
            e = field_errors(hst, want, cur)
            for k, v in e.items():
                report(f"moved by {shift / skin:.1f} skin, 1 step {k}", v, 5e-4)
            assert all(v < 5e-4 for v in e.values()), e
        assert sol.error_flags(stream=s) == 0


def test_kind_change_rebuilds(sphlib, oracle, cuda, report):
    """Boundary lists hold fluid neighbours only, so an upload that turns fluid particles into
    boundary particles rebuilds the lists; the step matches the oracle."""
    import torch
    from tmp_sph_gb300 import api, cases, solver as S
    from test_solver_gpu import field_errors
    st, p = cases.build("small", physics="config", dx=0.02, jitter=0.01)
    fl = np.nonzero(st["type"] == 1)[0]
    s = torch.cuda.Stream()
    with S.Solver(p, len(st["rho"])) as sol:
        sol.set_option(api.SPH_OPT_SKIN_PERMILLE, 100)
        hst = _pinned(st)
        sol.step_host(hst, 1, stream=s)
        base = sol.rebuild_count(stream=s)
        kinds = hst["type"].copy()
        kinds[fl[:50]] = 0
        cur = {k: hst[k].copy() for k in hst}
        cur["type"] = kinds
        want = oracle.run(oracle.params_like(p), cur, 1)
        hst["type"][...] = kinds
        sol.step_host(hst, 1, stream=s)
        assert sol.rebuild_count(stream=s) > base
        assert sol.error_flags(stream=s) == 0
    e = field_errors(hst, want, cur)
    for k, v in e.items():
        report(f"kind change, 1 step {k}", v, 5e-4)
    assert all(v < 5e-4 for v in e.values()), e


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_host_loop_other_precisions(sphlib, cuda, report, precision):
    """Mixed precision and FP64 take the same path; the FP32 host arrays round the state
    between calls, so the loop agrees with the resident run to that rounding."""
    import torch
    from tmp_sph_gb300 import api, cases, solver as S
    from gpu_util import perturbed
    st, p = cases.build("small", physics="config", dx=0.02, jitter=0.01)
    st = perturbed(st, vamp=1.0, ramp=0.0)
    steps = 6
    ref = _resident(st, p, steps, precision=precision)
    hst = _pinned(st)
    s = torch.cuda.Stream()
    with S.Solver(p, len(st["rho"]), precision=precision) as sol:
        sol.set_option(api.SPH_OPT_SKIN_PERMILLE, 100)
        for _ in range(steps):
            sol.step_host(hst, 1, stream=s)
        assert sol.error_flags(stream=s) == 0
    fl = st["type"] == 1
    e = rel_l2(hst["vel"][fl], ref["vel"][fl], floor=1e-3 * np.sqrt(fl.sum()))
    report(f"host loop {precision} vel vs resident", e, 1e-4)
    assert e < 1e-4
    assert np.array_equal(hst["type"], ref["type"])


def test_batched_reupload_keeps_order(sphlib, cuda):
    """Re-uploading the same instances (same offsets) continues the resident run bit for bit;
    different offsets start over from a fresh sort."""
    import torch
    from tmp_sph_gb300 import api, cases, solver as S
    states, p = cases.batch(2, dx=0.02, seed=5)
    n = sum(len(st["rho"]) for st in states)
    s = torch.cuda.Stream()
    outs = []
    for reupload in (False, True):
        with S.Solver(p, n) as sol:
            sol.set_option(api.SPH_OPT_SKIN_PERMILLE, 100)
            off = sol.upload_instances(states, stream=s)
            sol.step(3, stream=s)
            if reupload:
                mid = sol.download(stream=s)
                parts = [{k: mid[k][off[b]:off[b + 1]] for k in ("pos", "vel", "rho", "p", "type")}
                         for b in range(len(states))]
                sol.upload_instances(parts, stream=s)
            sol.step(3, stream=s)
            outs.append(sol.download(stream=s))
            assert sol.error_flags(stream=s) == 0
    for k in ("pos", "vel", "rho", "p", "type"):
        assert np.array_equal(outs[0][k], outs[1][k]), k
