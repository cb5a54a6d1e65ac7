"""Why the solver keeps velocity and rho - rho0 in FP32 rather than packed FP16.

A packed FP16 storage of the neighbour velocity and density perturbation would shrink the
records the neighbour passes gather, and is acceptable only if its error stays inside the
1e-3 relative-L2 tolerance.  This test measures it with the oracle on a developed flow (the
small dam break after 0.4 s, surge at ~2.8 m/s): the rates computed from a state whose
velocities and rho - rho0 are rounded to FP16 against the FP64 rates of the same state, next
to those of the FP32 state.  FP16 velocities put the rates off by more than the tolerance in
a single evaluation (neighbour velocity differences are a few per mille of the speed, the size
of FP16's spacing), three orders above FP32, so the variant is not built."""
from __future__ import annotations

import numpy as np
import pytest


def _rates(O, P, state, dtype):
    s = {k: np.array(state[k], dtype=np.int32 if k == "type" else dtype)
         for k in ("pos", "vel", "rho", "p", "type")}
    cl = O.cell_list(P, s)
    r = O.sph_ns(P, cl)
    inv = np.empty_like(cl["index"])
    inv[cl["index"]] = np.arange(len(inv))
    return {k: np.asarray(v, np.float64)[inv] for k, v in r.items()}


def _rel(a, b, mask):
    return float(np.linalg.norm((a - b)[mask]) / np.linalg.norm(b[mask]))


@pytest.mark.timeout(600)
def test_fp16_velocity_storage_exceeds_tolerance(oracle, report):
    from tmp_sph_gb300 import cases
    st, p = cases.build("small", physics="config", dx=0.04, jitter=0.01)
    P = oracle.params_like(p)
    oracle.set_threads(0)
    steps = int(round(0.4 / float(p.dt)))
    s64 = oracle.run(P, st, steps, dtype=np.float64)
    fl = s64["type"] == 1
    assert np.abs(s64["vel"][fl]).max() > 2.0  # a developed surge
    ref = _rates(oracle, P, s64, np.float64)
    r32 = _rates(oracle, P, s64, np.float32)
    half = dict(s64)
    half["vel"] = s64["vel"].astype(np.float16).astype(np.float64)
    half["rho"] = 1000.0 + (s64["rho"] - 1000.0).astype(np.float16).astype(np.float64)
    r16 = _rates(oracle, P, half, np.float32)
    e32 = max(_rel(r32["rho_dt"], ref["rho_dt"], fl), _rel(r32["vel_dt"], ref["vel_dt"], fl))
    e16 = max(_rel(r16["rho_dt"], ref["rho_dt"], fl), _rel(r16["vel_dt"], ref["vel_dt"], fl))
    report("rates from an FP32 state vs FP64 (developed flow)", e32, 1e-4)
    report("rates with FP16 velocity and rho - rho0 vs FP64 (developed flow)", e16, 1e-3)
    assert e32 < 1e-4
    assert e16 > 1e-3 and e16 > 100 * e32
