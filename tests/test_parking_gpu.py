"""GPU tests of escaped fluid particles (src/sph/sph_run.cu:437-447: a fluid particle outside
the escape box is parked with zero velocity).

park_inactive = 0 keeps the reference's behaviour: parked particles stay in the neighbour
search at the parking point, where they pile up in one cell.  park_inactive = 1 takes every
fluid particle outside the escape box out of the search: its key sorts after every cell, so it
is nobody's neighbour and walks no cells itself (the reference's later version marks such
particles with type 100 instead, opt_src_v4/sph/sph_run.cu:449).  Both are checked against
the oracle run with the same setting, on a case whose escape box cuts the water column in
half so thousands of particles escape in the first half step."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


def _case(park_inactive: int, dx: float = 0.02):
    from tmp_sph_gb300 import cases
    st, p = cases.build("small", physics="config", dx=dx, jitter=0.01)
    p.escape_max = type(p.escape_max)(p.escape_max[0], p.escape_max[1], 0.15)
    p.park_inactive = park_inactive
    return st, p


def _run(st, p, nsteps, skin=100, precision="fp32"):
    import torch
    from tmp_sph_gb300 import api, solver as S
    s = torch.cuda.Stream()
    with S.Solver(p, len(st["rho"]), precision=precision) as sol:
        sol.set_option(api.SPH_OPT_SKIN_PERMILLE, skin)
        sol.upload(st["pos"], st["vel"], st["rho"], st["p"], st["type"], stream=s)
        sol.step(nsteps, stream=s)
        out = sol.download(stream=s)
        out["flags"] = sol.error_flags(stream=s)
        _, out["stats"] = sol.probe(stream=s)
        out["rebuilds"] = sol.rebuild_count(stream=s)
    return out


@pytest.mark.parametrize("park_inactive", [0, 1])
def test_escaped_particles_match_oracle(sphlib, oracle, cuda, report, park_inactive):
    from tmp_sph_gb300 import api
    st, p = _case(park_inactive)
    steps = 3
    out = _run(st, p, steps)
    ref = oracle.run(oracle.params_like(p), st, steps)
    park = np.array(p.escape_park, np.float32)
    fl = st["type"] == 1
    parked = fl & np.all(ref["pos"] == park, axis=1)
    n_parked = int(parked.sum())
    report(f"park_inactive {park_inactive}: parked particles", n_parked)
    assert n_parked > 1000
    assert np.array_equal(np.all(out["pos"] == park, axis=1) & fl, parked)
    assert out["stats"]["parked"] == n_parked
    live = fl & ~parked
    e = {
        "disp": rel_l2(out["pos"][live] - st["pos"][live], ref["pos"][live] - st["pos"][live]),
        "vel": rel_l2(out["vel"][live], ref["vel"][live], floor=1e-3 * np.sqrt(live.sum())),
        "drho": rel_l2(out["rho"][live] - 1000.0, ref["rho"][live] - 1000.0),
    }
    for k, v in e.items():
        report(f"park_inactive {park_inactive}, {steps} steps {k}", v, 2e-4)
    assert all(v < 2e-4 for v in e.values()), e
    wl = st["type"] != 1
    np.testing.assert_allclose(out["p"][wl], ref["p"][wl], rtol=1e-3, atol=1.0)
    if park_inactive:
        # nobody searches the parking point, so no list overflows there
        assert out["flags"] == 0
    else:
        # thousands of parked particles share one cell: their lists overflow and they walk
        assert out["flags"] & ~api.SPH_FLAG_NEIGHBOR_OVERFLOW == 0


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_escaped_particles_other_precisions(sphlib, oracle, cuda, report, precision):
    st, p = _case(1)
    out = _run(st, p, 2, precision=precision)
    ref = oracle.run(oracle.params_like(p), st, 2)
    park = np.array(p.escape_park, np.float32)
    fl = st["type"] == 1
    parked = fl & np.all(ref["pos"] == park, axis=1)
    assert np.array_equal(np.all(out["pos"] == park, axis=1) & fl, parked)
    live = fl & ~parked
    e = rel_l2(out["vel"][live], ref["vel"][live], floor=1e-3 * np.sqrt(live.sum()))
    report(f"park_inactive {precision} 2 steps vel", e, 2e-4)
    assert e < 2e-4 and out["flags"] == 0


def test_inactive_particles_without_skin_or_list(sphlib, cuda):
    """Rebuilding every half step, and walking the cells without a list, give the same bits
    as each other with particles outside the search (the one-lane list passes and the walk
    skip them alike)."""
    from tmp_sph_gb300 import api
    import torch
    from tmp_sph_gb300 import solver as S
    st, p = _case(1)
    outs = []
    for use_list in (1, 0):
        s = torch.cuda.Stream()
        with S.Solver(p, len(st["rho"])) as sol:
            sol.set_option(api.SPH_OPT_SKIN_PERMILLE, 0)
            sol.set_option(api.SPH_OPT_NEIGHBOR_LIST, use_list)
            sol.set_option(api.SPH_OPT_LANES_PER_PARTICLE, 1)
            sol.upload(st["pos"], st["vel"], st["rho"], st["p"], st["type"], stream=s)
            sol.step(3, stream=s)
            outs.append(sol.download(stream=s))
            assert sol.error_flags(stream=s) == 0
    for k in ("pos", "vel", "rho", "p"):
        assert np.array_equal(outs[0][k], outs[1][k]), k


def test_inactive_batch_equals_solo(sphlib, cuda):
    """Batched instances with particles outside the search: each instance equals its solo run
    bit for bit (skin 0), the inactive particles of all instances sharing the sorted tail."""
    import torch
    from tmp_sph_gb300 import api, cases, solver as S
    states, p = cases.batch(2, dx=0.02, seed=7)
    p.escape_max = type(p.escape_max)(p.escape_max[0], p.escape_max[1], 0.12)
    p.park_inactive = 1
    n = sum(len(st["rho"]) for st in states)
    s = torch.cuda.Stream()
    with S.Solver(p, n) as sol:
        sol.set_option(api.SPH_OPT_SKIN_PERMILLE, 0)
        off = sol.upload_instances(states, stream=s)
        sol.step(3, stream=s)
        out = sol.download(stream=s)
        assert sol.error_flags(stream=s) == 0
    for b, st in enumerate(states):
        ref = _run(st, p, 3, skin=0)
        sl = slice(int(off[b]), int(off[b + 1]))
        for k in ("pos", "vel", "rho", "p", "type"):
            assert np.array_equal(out[k][sl], ref[k]), (b, k)


def test_inactive_host_loop_equals_resident_run(sphlib, cuda):
    """Uploads into the current order keep the inactive tail: a loop of one-step host calls
    gives the bits of one resident run."""
    import torch
    from tmp_sph_gb300 import api, solver as S
    st, p = _case(1)
    ref = _run(st, p, 6)
    hst = {k: torch.from_numpy(np.ascontiguousarray(st[k])).pin_memory().numpy()
           for k in ("pos", "vel", "rho", "p", "type")}
    s = torch.cuda.Stream()
    with S.Solver(p, len(st["rho"])) as sol:
        sol.set_option(api.SPH_OPT_SKIN_PERMILLE, 100)
        for _ in range(6):
            sol.step_host(hst, 1, stream=s)
        assert sol.error_flags(stream=s) == 0
    for k in ("pos", "vel", "rho", "p"):
        assert np.array_equal(hst[k], ref[k]), k
