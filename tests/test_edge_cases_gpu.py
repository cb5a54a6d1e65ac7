"""Edge cases of the resident solver on the GPU: an empty state, a single particle, walls only,
a crowd of particles in one cell (their lists overflow and they walk the cells), particles on
cell faces and grid edges, and a batch of very different instances (one particle, walls only,
a full dam break).  Each is checked against the oracle or against the same instances run
alone."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


def _state(pos, typ, vel=None):
    pos = np.ascontiguousarray(pos, np.float32)
    n = len(pos)
    return {"pos": pos,
            "vel": np.zeros((n, 3), np.float32) if vel is None else np.ascontiguousarray(vel, np.float32),
            "rho": np.full(n, 1000.0, np.float32), "p": np.zeros(n, np.float32),
            "type": np.ascontiguousarray(typ, np.int32)}


def _run(st, p, nsteps, skin=100, capacity=None):
    import torch
    from tmp_sph_gb300 import api, solver as S
    n = len(st["rho"])
    s = torch.cuda.Stream()
    with S.Solver(p, capacity if capacity is not None else max(n, 1)) as sol:
        sol.set_option(api.SPH_OPT_SKIN_PERMILLE, skin)
        sol.upload(st["pos"], st["vel"], st["rho"], st["p"], st["type"], stream=s)
        sol.step(nsteps, stream=s)
        out = sol.download(stream=s)
        out["flags"] = sol.error_flags(stream=s)
        out["steps"] = sol.steps_taken()
    return out


def _params():
    from tmp_sph_gb300 import cases
    return cases.build("small", physics="config", dx=0.02, jitter=0.01)


def test_empty_state(sphlib, cuda):
    _, p = _params()
    out = _run(_state(np.zeros((0, 3)), np.zeros(0)), p, 3, capacity=16)
    assert out["flags"] == 0 and out["steps"] == 3 and len(out["rho"]) == 0


def test_single_particle_falls_freely(sphlib, oracle, cuda):
    """No neighbours: the midpoint scheme integrates gravity exactly as the reference does."""
    _, p = _params()
    st = _state([[0.5, 0.25, 0.3]], [1])
    out = _run(st, p, 10)
    ref = oracle.run(oracle.params_like(p), st, 10)
    assert out["flags"] == 0
    # the reference forms x + v dt / 2.0 in double, the solver in float: a few ulp apart
    ulp = np.spacing(np.abs(ref["pos"]).astype(np.float32))
    assert np.all(np.abs(out["pos"] - ref["pos"]) <= 4 * ulp)
    np.testing.assert_allclose(out["vel"], ref["vel"], rtol=1e-5)
    assert out["vel"][0, 2] < 0 and out["pos"][0, 2] < 0.3


def test_walls_only(sphlib, oracle, cuda):
    """Boundary particles without fluid keep their positions; their extrapolated pressure has
    no fluid to come from."""
    st, p = _params()
    wl = st["type"] != 1
    walls = {k: v[wl].copy() for k, v in st.items() if isinstance(v, np.ndarray)}
    out = _run(walls, p, 3)
    ref = oracle.run(oracle.params_like(p), walls, 3)
    assert out["flags"] == 0
    assert np.array_equal(out["pos"], walls["pos"])
    np.testing.assert_allclose(out["p"], ref["p"], atol=1e-3)
    np.testing.assert_allclose(out["rho"], ref["rho"], rtol=1e-6)


def test_crowd_in_one_cell(sphlib, oracle, cuda, report):
    """300 fluid particles packed within 0.3 dx: each has more neighbours than its list holds,
    raises SPH_FLAG_NEIGHBOR_OVERFLOW and walks the cells; one step matches the oracle."""
    from tmp_sph_gb300 import api
    from gpu_util import perturbed
    st, p = _params()
    st = perturbed(st, vamp=0.3, ramp=0.02)
    rng = np.random.default_rng(4)
    fl = np.nonzero(st["type"] == 1)[0][:300]
    st["pos"][fl] = (np.array([0.2, 0.25, 0.1]) + rng.uniform(0, 0.3 * p.dx, (300, 3))).astype(np.float32)
    out = _run(st, p, 1)
    ref = oracle.run(oracle.params_like(p), st, 1)
    assert out["flags"] & api.SPH_FLAG_NEIGHBOR_OVERFLOW
    assert out["flags"] & ~api.SPH_FLAG_NEIGHBOR_OVERFLOW == 0
    f = st["type"] == 1
    e = rel_l2(out["vel"][f], ref["vel"][f], floor=1e-3 * np.sqrt(f.sum()))
    report("crowd of 300 in one cell, 1 step vel", e, 1e-4)
    assert e < 1e-4
    e = rel_l2(out["rho"][f] - 1000.0, ref["rho"][f] - 1000.0)
    report("crowd of 300 in one cell, 1 step rho - rho0", e, 1e-4)
    assert e < 1e-4


def test_cell_faces_and_grid_edges(sphlib, oracle, cuda, report):
    """Fluid particles exactly on cell faces of the solver's grid and of the reference grid,
    and on the lower grid corner, hash consistently (no flag) and step like the oracle."""
    from tmp_sph_gb300 import api
    st, p = _params()
    fl = np.nonzero(st["type"] == 1)[0]
    g0 = np.array(p.grid_min[:], np.float32)
    cell_ref = np.float32(p.cell_size)
    cell_res = np.float32(p.kh * 1.1)
    faces = [g0 + cell_ref * np.array([10, 5, 3], np.float32),
             g0 + cell_res * np.array([10, 5, 3], np.float32),
             g0 + cell_ref * np.array([20, 7, 2], np.float32)]
    for k, xyz in enumerate(faces):
        st["pos"][fl[k]] = xyz
    out = _run(st, p, 1)
    ref = oracle.run(oracle.params_like(p), st, 1)
    assert out["flags"] == 0
    f = st["type"] == 1
    e = rel_l2(out["vel"][f], ref["vel"][f], floor=1e-3 * np.sqrt(f.sum()))
    report("particles on cell faces, 1 step vel", e, 2e-5)
    assert e < 2e-5
    # on the lower corner of the grid itself: still inside, no flag
    st2, _ = _params()
    st2["pos"][fl[0]] = g0
    out2 = _run(st2, p, 1)
    assert out2["flags"] & api.SPH_FLAG_OUT_OF_GRID == 0


def test_ragged_batch_equals_solo(sphlib, cuda):
    """Instances of 1 particle, walls only and a full dam break, batched: each equals its solo
    run bit for bit (skin 0: the same rebuild schedule)."""
    import torch
    from tmp_sph_gb300 import api, solver as S
    st, p = _params()
    wl = st["type"] != 1
    walls = {k: v[wl].copy() for k, v in st.items() if isinstance(v, np.ndarray)}
    one = _state([[0.3, 0.2, 0.35]], [1])
    states = [one, walls, {k: v for k, v in st.items() if isinstance(v, np.ndarray)}, one]
    n = sum(len(s_["rho"]) for s_ in states)
    s = torch.cuda.Stream()
    with S.Solver(p, n) as sol:
        sol.set_option(api.SPH_OPT_SKIN_PERMILLE, 0)
        off = sol.upload_instances(states, stream=s)
        sol.step(4, stream=s)
        out = sol.download(stream=s)
        assert sol.error_flags(stream=s) == 0
    for b, sb in enumerate(states):
        ref = _run(sb, p, 4, skin=0)
        sl = slice(int(off[b]), int(off[b + 1]))
        for k in ("pos", "vel", "rho", "p", "type"):
            assert np.array_equal(out[k][sl], ref[k]), (b, k)


def test_reupload_with_other_count(sphlib, cuda):
    """An upload of a different number of particles after stepping starts over (fresh sort and
    lists) and matches a fresh solver."""
    import torch
    from tmp_sph_gb300 import api, solver as S
    st, p = _params()
    half = {k: v[: len(v) // 2].copy() for k, v in st.items() if isinstance(v, np.ndarray)}
    s = torch.cuda.Stream()
    with S.Solver(p, len(st["rho"])) as sol:
        sol.upload(st["pos"], st["vel"], st["rho"], st["p"], st["type"], stream=s)
        sol.step(2, stream=s)
        sol.upload(half["pos"], half["vel"], half["rho"], half["p"], half["type"], stream=s)
        sol.step(2, stream=s)
        out = sol.download(stream=s)
        assert sol.error_flags(stream=s) == 0
    ref = _run(half, p, 2, capacity=len(st["rho"]))
    for k in ("pos", "vel", "rho", "p"):
        assert np.array_equal(out[k], ref[k]), k
