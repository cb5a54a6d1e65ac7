"""GPU parity of the cell list: hash, stable radix sort, reorder (cell start/end + gather) and
recover, bit-for-bit against the oracle (src/lib/mesh.cu:6-194) on the same inputs."""
from __future__ import annotations

import numpy as np
import pytest

from gpu_util import dev, host

pytestmark = pytest.mark.gpu


def _state(name="small", physics="reference", **kw):
    from tmp_sph_gb300 import cases
    return cases.build(name, physics=physics, **kw)


def gpu_cell_list(p, st, cuda, key_bits=32):
    import torch
    from tmp_sph_gb300 import solver as S
    n = len(st["rho"])
    pos = dev(st["pos"], cuda)
    h = torch.empty(n, dtype=torch.int32, device=cuda)
    idx = torch.empty(n, dtype=torch.int32, device=cuda)
    S.calc_hash(p, pos, h, idx, n)
    h_unsorted = host(h).copy()
    S.sort_particles(h, idx, n, key_bits=key_bits)
    out = {k: torch.empty_like(dev(st[k], cuda)) for k in ("pos", "vel", "rho", "p", "type")}
    cs = torch.empty(p.num_cells, dtype=torch.int32, device=cuda)
    ce = torch.full((p.num_cells,), -7, dtype=torch.int32, device=cuda)
    S.reorder(p, pos, dev(st["vel"], cuda), dev(st["rho"], cuda), dev(st["p"], cuda),
              dev(st["type"], cuda), None, out["pos"], out["vel"], out["rho"], out["p"],
              out["type"], None, h, idx, cs, ce, n)
    res = {k: host(v) for k, v in out.items()}
    res.update(hash=host(h), index=host(idx), cell_start=host(cs), cell_end=host(ce),
               hash_unsorted=h_unsorted)
    return res


@pytest.mark.parametrize("case,physics,kw", [
    ("small", "reference", dict(jitter=0.01)),
    ("small", "config", dict()),
    ("refcase", "reference", dict(dx=0.02, jitter=0.02)),
    ("obstacle", "config", dict(dx=0.02, jitter=0.01)),
])
def test_cell_list_bit_exact(sphlib, oracle, cuda, case, physics, kw):
    st, p = _state(case, physics, **kw)
    P = oracle.params_like(p)
    ref = oracle.cell_list(P, st)
    href, _ = oracle.calc_hash(P, st["pos"])
    for bits in (32, 0):
        g = gpu_cell_list(p, st, cuda, key_bits=bits or max(1, int(np.ceil(np.log2(p.num_cells)))))
        assert np.array_equal(g["hash_unsorted"], href)
        assert np.array_equal(g["hash"], ref["hash"])
        assert np.array_equal(g["index"], ref["index"])
        assert np.array_equal(g["cell_start"], ref["cell_start"])
        occ = ref["cell_start"] >= 0
        assert np.array_equal(g["cell_end"][occ], ref["cell_end"][occ])
        for k in ("pos", "vel", "rho", "p", "type"):
            assert np.array_equal(g[k], ref[k]), k


def test_hash_on_cell_faces(sphlib, oracle, cuda):
    """Positions exactly on cell faces (p = min + k*gridSize in float32) and one cell-width
    either side hash exactly as the reference's float expression."""
    import torch
    from tmp_sph_gb300 import solver as S
    _, p = _state("small", "reference")
    P = oracle.params_like(p)
    ks = np.arange(0, p.grid_dim[0], dtype=np.float32)
    faces = np.float32(p.grid_min[0]) + ks * np.float32(p.cell_size)
    eps = np.spacing(faces)
    xs = np.concatenate([faces, faces + eps, faces - eps]).astype(np.float32)
    xs = xs[(xs > p.grid_min[0]) & (xs < p.grid_max[0])]
    pos = np.stack([xs, np.full_like(xs, 0.25), np.full_like(xs, 0.3)], 1).astype(np.float32)
    href, _ = oracle.calc_hash(P, np.ascontiguousarray(pos))
    n = len(xs)
    h = torch.empty(n, dtype=torch.int32, device=cuda)
    idx = torch.empty(n, dtype=torch.int32, device=cuda)
    S.calc_hash(p, dev(pos, cuda), h, idx, n)
    assert np.array_equal(host(h), href)
    assert np.array_equal(host(idx), np.arange(n))


@pytest.mark.parametrize("n", [1, 2, 31, 4095, 4096, 4097, 100003, 1 << 20])
@pytest.mark.parametrize("kind", ["small_range", "full_int32", "cells22"])
def test_radix_sort_stable(sphlib, cuda, n, kind):
    """sortParticles semantics: ascending signed keys, equal keys keep their input order."""
    import torch
    from tmp_sph_gb300 import solver as S
    rng = np.random.default_rng(n)
    if kind == "small_range":
        keys, bits = rng.integers(0, 40, n), 6
    elif kind == "full_int32":
        keys, bits = rng.integers(-2**31, 2**31 - 1, n, endpoint=True), 32
    else:
        keys = np.sort(rng.integers(0, 2**22, n))
        keys[rng.integers(0, n, n // 20 + 1)] += 1  # nearly sorted, like a cell list
        keys = np.minimum(keys, 2**22 - 1)
        bits = 22
    keys = keys.astype(np.int32)
    vals = rng.permutation(n).astype(np.int32)
    order = np.argsort(keys, kind="stable")
    for kb in sorted({bits, 32}):
        h = dev(keys, cuda)
        v = dev(vals, cuda)
        S.sort_particles(h, v, n, key_bits=kb)
        assert np.array_equal(host(h), keys[order]), kb
        assert np.array_equal(host(v), vals[order]), kb


def test_sort_scratch_too_small_is_an_error(sphlib, cuda):
    import torch
    from tmp_sph_gb300 import api
    n = 5000
    h = torch.zeros(n, dtype=torch.int32, device=cuda)
    v = torch.zeros(n, dtype=torch.int32, device=cuda)
    small = torch.empty(16, dtype=torch.uint8, device=cuda)
    st = api.lib().sph_sort_particles(h.data_ptr(), v.data_ptr(), n, 32, small.data_ptr(), 16, None)
    assert st == api.SPH_ERR_SCRATCH


def test_edge_cases(sphlib, oracle, cuda):
    """One particle; every particle in one cell; empty first and last cells."""
    _, p = _state("small", "reference")
    P = oracle.params_like(p)
    c = np.array([0.5, 0.25, 0.3], np.float32)
    for pos in (c[None, :],
                np.repeat(c[None, :], 300, 0) + np.float32(1e-4) * np.arange(300, dtype=np.float32)[:, None] / 300,
                np.array([[-0.05, -0.05, -0.05], [1.05, 0.55, 0.65], [0.5, 0.25, 0.3]], np.float32)):
        n = len(pos)
        st = {"pos": np.ascontiguousarray(pos, np.float32), "vel": np.zeros((n, 3), np.float32),
              "rho": np.full(n, 1000, np.float32), "p": np.zeros(n, np.float32),
              "type": np.ones(n, np.int32)}
        ref = oracle.cell_list(P, st)
        g = gpu_cell_list(p, st, cuda)
        for k in ("hash", "index", "cell_start"):
            assert np.array_equal(g[k], ref[k]), k
        occ = ref["cell_start"] >= 0
        assert np.array_equal(g["cell_end"][occ], ref["cell_end"][occ])


def test_zero_particles(sphlib, cuda):
    import torch
    from tmp_sph_gb300 import solver as S
    _, p = _state("small", "reference")
    z = torch.empty(0, dtype=torch.int32, device=cuda)
    zf = torch.empty(0, dtype=torch.float32, device=cuda)
    S.calc_hash(p, zf, z, z, 0)
    S.sort_particles(z, z, 0)
    cs = torch.zeros(p.num_cells, dtype=torch.int32, device=cuda)
    ce = torch.zeros(p.num_cells, dtype=torch.int32, device=cuda)
    S.reorder(p, zf, zf, zf, zf, z, None, zf, zf, zf, zf, z, None, z, z, cs, ce, 0)
    assert (host(cs) == -1).all()


def test_recover_inverts_reorder(sphlib, oracle, cuda):
    import torch
    from tmp_sph_gb300 import solver as S
    st, p = _state("small", "reference", jitter=0.01)
    n = len(st["rho"])
    g = gpu_cell_list(p, st, cuda)
    outs = {k: torch.zeros_like(dev(st[k], cuda)) for k in ("pos", "vel", "rho", "p", "type")}
    S.recover(outs["pos"], outs["vel"], outs["rho"], outs["p"], n, dev(g["index"], cuda),
              outs["type"], None, dev(g["pos"], cuda), dev(g["vel"], cuda), dev(g["rho"], cuda),
              dev(g["p"], cuda), dev(g["type"], cuda), None)
    for k in outs:
        assert np.array_equal(host(outs[k]), st[k]), k
