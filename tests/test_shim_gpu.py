"""GPU test of the reference-signature shim: one full step of the reference's own step loop
(src/sph/sph_run.cu:285-336) driven through the C++-linkage functions calcHash,
sortParticles, reorder, SPH_NS_simpleversion, PC_prediction, PC_correction and recover that
the library exports with the reference's exact signatures, compared with the oracle running
the same loop.  Same dataflow, same summation order: agreement to a few float ulps."""
from __future__ import annotations

import ctypes as C
import subprocess

import numpy as np
import pytest

from conftest import rel_l2
from gpu_util import dev, host

pytestmark = pytest.mark.gpu


def shim_functions():
    from tmp_sph_gb300 import api
    raw = subprocess.run(["nm", "-D", "--defined-only", api.LIB_PATH], capture_output=True,
                         text=True, check=True).stdout.splitlines()
    dem = subprocess.run(["nm", "-D", "--defined-only", "-C", api.LIB_PATH], capture_output=True,
                         text=True, check=True).stdout.splitlines()
    table = {}
    for a, b in zip(raw, dem):
        m, d = a.split()[-1], b.split(None, 2)[-1]
        table[d.split("(")[0]] = m
    L = api.lib()
    P = C.c_void_p
    sig = {
        "calcHash": [P, P, P, C.c_int],
        "sortParticles": [P, P, C.c_int],
        "reorder": [P] * 16 + [C.c_int, P],
        "recover": [P, P, P, P, C.c_int] + [P] * 9,
        "SPH_NS_simpleversion": [P] * 9 + [C.c_int, P, C.c_int, P, P, P],
        "PC_prediction": [P] * 11 + [C.c_int, P],
        "PC_correction": [P] * 11 + [C.c_int, P],
    }
    fns = {}
    for name, args in sig.items():
        f = getattr(L, table[name])
        f.restype = None
        f.argtypes = args
        fns[name] = f
    return fns


@pytest.mark.parametrize("physics", ["reference", "config"])
def test_reference_step_loop_through_shim(sphlib, oracle, cuda, report, physics):
    import torch
    from tmp_sph_gb300 import api, cases
    st, p = cases.build("small", physics=physics, dx=0.02, jitter=0.01)
    n = len(st["rho"])
    f = shim_functions()
    api.call("sph_shim_set_params", C.byref(p))
    d = {k: dev(st[k], cuda) for k in ("pos", "vel", "rho", "p", "type")}
    d["zone"] = torch.zeros(n, dtype=torch.int32, device=cuda)
    s = {k: torch.empty_like(v) for k, v in d.items()}
    ix = {k: torch.empty(n, dtype=torch.int32, device=cuda) for k in ("hash", "index")}
    cs = torch.empty(p.num_cells, dtype=torch.int32, device=cuda)
    ce = torch.empty(p.num_cells, dtype=torch.int32, device=cuda)
    rdt = torch.zeros(n, device=cuda)
    vdt = torch.zeros((n, 3), device=cuda)
    dofv, rs, ws = (torch.zeros(n, device=cuda) for _ in range(3))
    tmp = {"pos": torch.zeros((n, 3), device=cuda), "vel": torch.zeros((n, 3), device=cuda),
           "rho": torch.zeros(n, device=cuda)}
    ref_params = api.params_to_reference(p)
    P_ = lambda t: t.data_ptr()
    torch.cuda.synchronize()
    for half in range(2):
        f["calcHash"](P_(d["pos"]), P_(ix["hash"]), P_(ix["index"]), n)
        f["sortParticles"](P_(ix["hash"]), P_(ix["index"]), n)
        f["reorder"](P_(d["pos"]), P_(d["vel"]), P_(d["rho"]), P_(d["p"]), P_(d["type"]),
                     P_(d["zone"]), P_(s["pos"]), P_(s["vel"]), P_(s["rho"]), P_(s["p"]),
                     P_(s["type"]), P_(s["zone"]), P_(ix["hash"]), P_(ix["index"]), P_(cs), P_(ce),
                     n, C.addressof(ref_params))
        f["SPH_NS_simpleversion"](P_(s["pos"]), P_(s["vel"]), P_(s["rho"]), P_(s["p"]),
                                  P_(s["type"]), P_(rdt), P_(vdt), P_(cs), P_(ce), n,
                                  P_(ix["hash"]), 0, P_(dofv), P_(rs), P_(ws))
        pc = f["PC_prediction"] if half == 0 else f["PC_correction"]
        pc(P_(s["pos"]), P_(s["vel"]), P_(s["rho"]), P_(s["p"]), P_(rdt), P_(vdt), P_(ix["hash"]),
           P_(ix["index"]), P_(tmp["pos"]), P_(tmp["vel"]), P_(tmp["rho"]), n, P_(s["type"]))
        f["recover"](P_(d["pos"]), P_(d["vel"]), P_(d["rho"]), P_(d["p"]), n, P_(ix["index"]),
                     P_(d["type"]), P_(d["zone"]), P_(s["pos"]), P_(s["vel"]), P_(s["rho"]),
                     P_(s["p"]), P_(s["type"]), P_(s["zone"]))
    torch.cuda.synchronize()
    out = {k: host(v) for k, v in d.items()}
    ref = oracle.run(oracle.params_like(p), st, 1)
    fl = st["type"] == 1
    e_x = rel_l2(out["pos"][fl] - st["pos"][fl], ref["pos"][fl] - st["pos"][fl])
    e_v = rel_l2(out["vel"][fl], ref["vel"][fl], floor=1e-3 * np.sqrt(fl.sum()))
    e_r = rel_l2(out["rho"][fl] - 1000, ref["rho"][fl] - 1000)
    report(f"shim step {physics} disp", e_x, 2e-5)
    report(f"shim step {physics} vel", e_v, 2e-5)
    report(f"shim step {physics} drho", e_r, 2e-5)
    assert e_x < 2e-5 and e_v < 2e-5 and e_r < 2e-5
    assert np.array_equal(out["type"], st["type"])
    api.call("sph_shim_release")
