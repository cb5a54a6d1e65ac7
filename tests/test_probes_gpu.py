"""GPU tests of the on-device probes and FP64 reductions (sph_probe_read) against the same
quantities computed with numpy from the downloaded state, in all three precisions.

The reference computes its gauges on the host from a full copy of the state
(src/io/io.cu:236-279): water height = largest z of fluid particles within 1.5 dx of a vertical
line, with a z cap for one gauge.  The heights and the surge front are extremes of the same
numbers and must match exactly; sums are FP64 in a different order (1e-12)."""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def wendland(p, r):
    q = r / p.h
    t = 1.0 - 0.5 * q
    return p.adh * t ** 4 * (2.0 * q + 1.0)


@pytest.mark.parametrize("precision", ["fp32", "mixed", "fp64"])
def test_probes_match_host_scan(sphlib, cuda, report, precision):
    import torch
    from tmp_sph_gb300 import api, cases, solver as S
    from gpu_util import perturbed
    st, p = cases.build("small", physics="config", dx=0.02, jitter=0.01)
    st = perturbed(st, vamp=0.5, ramp=0.01)
    n = len(st["rho"])
    s = torch.cuda.Stream()
    dx = float(p.dx)
    probes = [
        (api.SPH_PROBE_PRESSURE, 0.2, 0.25, 0.05, 0.0, 0.0),
        (api.SPH_PROBE_PRESSURE, 0.39, 0.02, 0.28, 0.0, 0.0),
        (api.SPH_PROBE_PRESSURE, 0.9, 0.25, 0.5, 0.0, 0.0),   # no fluid there
        (api.SPH_PROBE_HEIGHT, 0.2, 0.25, 0.0, 1.5 * dx, 0.0),
        (api.SPH_PROBE_HEIGHT, 0.2, 0.25, 0.0, 1.5 * dx, 0.2),
        (api.SPH_PROBE_FRONT, 0.0, 0.0, 0.0, 0.0, 0.0),
    ]
    with S.Solver(p, n, precision=precision) as sol:
        sol.upload(st["pos"], st["vel"], st["rho"], st["p"], st["type"], stream=s)
        sol.step(4, stream=s)
        vals, stats = sol.probe(probes, cfl=0.25, stream=s)
        out = sol.download_f64(stream=s)
    fl = st["type"] == 1
    x, v, rho, pr = out["pos"][fl], out["vel"][fl], out["rho"][fl], out["p"][fl]
    m = float(p.mass)
    assert stats["fluid"] == int(fl.sum()) and stats["parked"] == 0
    np.testing.assert_allclose(stats["mass"], m * fl.sum(), rtol=1e-12)
    np.testing.assert_allclose(stats["kinetic"], 0.5 * m * (v ** 2).sum(), rtol=1e-10)
    np.testing.assert_allclose(stats["potential"], -m * float(p.gravity) * x[:, 2].sum(),
                               rtol=1e-10)
    speed = np.sqrt((v ** 2).sum(axis=1)).max()
    np.testing.assert_allclose(stats["max_speed"], speed, rtol=1e-12)
    assert stats["rho_min"] == rho.min() and stats["rho_max"] == rho.max()
    assert stats["front_x"] == x[:, 0].max()
    np.testing.assert_allclose(stats["cfl_dt"], 0.25 * float(p.h) / (float(p.cs) + speed),
                               rtol=1e-12)
    # pressure probes: Shepard average over fluid within kh
    for q in range(3):
        c = np.array(probes[q][1:4], np.float32).astype(np.float64)
        r = np.sqrt(((x - c) ** 2).sum(axis=1))
        near = r < float(p.kh)
        want = (pr[near] * wendland(p, r[near])).sum() / wendland(p, r[near]).sum() \
            if near.any() else 0.0
        report(f"{precision} pressure probe {q}", vals[q] - want)
        np.testing.assert_allclose(vals[q], want, rtol=1e-9, atol=1e-9)
    assert vals[2] == 0.0
    # height gauges and the front
    for q in (3, 4):
        _, gx, gy, _, rad, zmax = probes[q]
        gx, gy, rad, zmax = (float(np.float32(t)) for t in (gx, gy, rad, zmax))
        col = (np.abs(x[:, 0] - gx) < rad) & (np.abs(x[:, 1] - gy) < rad)
        if zmax > 0:
            col &= x[:, 2] < zmax
        assert vals[q] == (x[col, 2].max() if col.any() else 0.0)
    assert vals[4] < 0.2 <= vals[3]
    assert vals[5] == x[:, 0].max()


def test_probe_arguments(sphlib, cuda):
    import torch
    from tmp_sph_gb300 import api, cases, solver as S
    st, p = cases.build("small", physics="config", dx=0.04)
    n = len(st["rho"])
    with S.Solver(p, n) as sol:
        lib = api.lib()
        arr = (api.SphProbe * 33)()
        vals = (ctypes.c_double * 33)()
        assert lib.sph_probe_read(sol.handle, arr, 1, vals, 0.25, None, None) == api.SPH_ERR_STATE
        sol.upload(st["pos"], st["vel"], st["rho"], st["p"], st["type"],
                   stream=torch.cuda.current_stream())
        assert lib.sph_probe_read(sol.handle, arr, 33, vals, 0.25, None, None) == api.SPH_ERR_ARG
        assert lib.sph_probe_read(sol.handle, None, 1, vals, 0.25, None, None) == api.SPH_ERR_ARG
        assert lib.sph_probe_read(sol.handle, arr, 0, None, 0.25, None, None) == api.SPH_OK
