"""CPU tests of the oracle itself: the cell list it builds obeys the reference's contract
(stable sort, cell ranges), its float and double instantiations agree, and it reproduces
physical invariants of the dam break.  Golden-vector pins against the reference's own kernels
live in test_golden.py."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import rel_l2


def small_state(dx=0.02, physics="reference", **kw):
    from tmp_sph_gb300 import cases
    st, p = cases.build("small", physics=physics, dx=dx, **kw)
    return st, p


def test_sort_is_stable_and_signed(oracle):
    rng = np.random.default_rng(1)
    for n in (0, 1, 2, 17, 4096, 100003):
        h = rng.integers(-50, 50, n).astype(np.int32)
        idx = np.arange(n, dtype=np.int32)
        ref = np.argsort(h, kind="stable").astype(np.int32)
        hh, ii = h.copy(), idx.copy()
        oracle.sort_particles(hh, ii)
        assert np.array_equal(ii, ref) and np.array_equal(hh, h[ref])
    h = np.array([2**31 - 1, -2**31, 0, -1, 5], np.int32)
    i = np.arange(5, dtype=np.int32)
    oracle.sort_particles(h, i)
    assert list(h) == sorted([2**31 - 1, -2**31, 0, -1, 5])


def test_cell_list_contract(sphlib, oracle):
    st, p = small_state(jitter=0.01)
    P = oracle.params_like(p)
    c = oracle.cell_list(P, st)
    h, idx = c["hash"], c["index"]
    assert (np.diff(h) >= 0).all()
    # stable: equal hashes keep ascending original index
    same = np.diff(h) == 0
    assert (np.diff(idx)[same] > 0).all()
    cs, ce = c["cell_start"], c["cell_end"]
    occupied = np.unique(h)
    assert (cs[np.setdiff1d(np.arange(P.num_cells), occupied)] == -1).all()
    for cell in occupied[:: max(1, len(occupied) // 500)]:
        s, e = cs[cell], ce[cell]
        assert (h[s:e] == cell).all()
        assert (s == 0 or h[s - 1] != cell) and (e == len(h) or h[e] != cell)
    # gathered arrays follow the permutation
    assert np.array_equal(c["pos"], st["pos"][idx])
    assert np.array_equal(c["type"], st["type"][idx])


def test_hash_matches_numpy_float32(sphlib, oracle):
    """floorf((p - min)/gridSize) in float32, z-major linear hash (src/lib/mesh.cu:6-23)."""
    st, p = small_state(jitter=0.01)
    P = oracle.params_like(p)
    h, _ = oracle.calc_hash(P, st["pos"])
    pos = st["pos"]
    g = [np.floor((pos[:, c] - np.float32(P.grid_min[c])) / np.float32(P.cell_size)).astype(np.int64)
         for c in range(3)]
    ref = g[2] * P.grid_dim[0] * P.grid_dim[1] + g[1] * P.grid_dim[0] + g[0]
    assert np.array_equal(h, ref.astype(np.int32))


def test_f32_f64_agree_one_ns(sphlib, oracle, report):
    st, p = small_state(jitter=0.01)
    P = oracle.params_like(p)
    s32 = oracle.cell_list(P, st)
    st64 = {k: (v.astype(np.float64) if v.dtype == np.float32 else v) for k, v in st.items()
            if isinstance(v, np.ndarray)}
    s64 = oracle.cell_list(P, st64)
    assert np.array_equal(s32["index"], s64["index"])
    r32 = oracle.sph_ns(P, s32)
    r64 = oracle.sph_ns(P, s64)
    fl = s32["type"] == 1
    e_a = rel_l2(r32["vel_dt"][fl], r64["vel_dt"][fl], floor=9.81 * np.sqrt(fl.sum()))
    e_r = rel_l2(r32["rho_dt"][fl], r64["rho_dt"][fl])
    report("oracle f32 vs f64 vel_dt", e_a)
    report("oracle f32 vs f64 rho_dt", e_r)
    assert e_a < 1e-3 and e_r < 1e-2


def test_hydrostatic_column_is_near_rest(sphlib, oracle):
    """Dam break starts near hydrostatic balance: after a few steps the fluid speed is far
    below the collapse speed sqrt(g H) and the density stays near rho0."""
    st, p = small_state(dx=0.02)
    P = oracle.params_like(p)
    out = oracle.run(P, st, 5)
    fl = st["type"] == 1
    vmax = np.abs(out["vel"][fl]).max()
    assert np.isfinite(out["pos"]).all()
    assert vmax < 0.5 * np.sqrt(9.81 * 0.3)
    assert np.abs(out["rho"][fl] / 1000 - 1).max() < 0.05
    # walls do not move
    assert np.array_equal(out["pos"][~fl], st["pos"][~fl])


def test_mass_and_count_conserved(sphlib, oracle):
    st, p = small_state(dx=0.02)
    P = oracle.params_like(p)
    out = oracle.run(P, st, 3)
    assert np.array_equal(out["type"], st["type"])
    assert np.isfinite(out["rho"]).all()


def test_escape_parks_particle(sphlib, oracle):
    """A fluid particle outside the escape box is parked (src/sph/sph_run.cu:437-447)."""
    st, p = small_state(dx=0.04)
    P = oracle.params_like(p)
    i = int(np.nonzero(st["type"] == 1)[0][0])
    st["pos"][i] = (0.5, 0.25, P.escape_max[2] + 0.01)
    out = oracle.run(P, st, 1)
    assert np.allclose(out["pos"][i], P.escape_park, atol=0)
    assert (out["vel"][i] == 0).all() and out["p"][i] == 0 and out["rho"][i] == P.rho0


@pytest.mark.parametrize("threads", [1, 3])
def test_openmp_deterministic(sphlib, oracle, threads):
    st, p = small_state(dx=0.04)
    P = oracle.params_like(p)
    oracle.set_threads(threads)
    a = oracle.run(P, st, 2)
    oracle.set_threads(0)
    b = oracle.run(P, st, 2)
    for k in ("pos", "vel", "rho", "p"):
        assert np.array_equal(a[k], b[k])


@pytest.mark.parametrize("name", ["small", "precision", "large", "obstacle"])
def test_oracle_workload_matches_product_workload(sphlib, oracle, name):
    """The oracle side builds every benchmark workload by itself (its own MT19937-64 generator
    and parameter derivation, so bench.py's reference leg loads no product library) and gets
    the product generator's state and the product's parameters bit for bit, jitter included."""
    from oracle import workload as W
    from tmp_sph_gb300 import cases
    a, pa = W.build(name)
    b, pb = cases.build(name)
    for k in ("pos", "vel", "rho", "p", "type"):
        assert a[k].dtype == b[k].dtype and np.array_equal(a[k], b[k]), (name, k)
    assert (a["n_fluid"], a["n_boundary"]) == (b["n_fluid"], b["n_boundary"])
    assert pa.as_dict() == oracle.params_like(pb).as_dict()
    if name == "large":
        assert len(a["rho"]) == 4963548 and a["n_fluid"] == 3840000
