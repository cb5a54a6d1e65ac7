"""GPU parity of the two neighbour passes (SPH_NS_simpleversion, src/equation/ns.cu:5-249)
against the oracle on identical sorted inputs.

Tolerances (relative L2 over fluid rows, FP32): the GPU evaluates the same sums in the same
order (z, y, x cells, sorted slots) with the kernel gradient in its factored form
c_fr (1 - q/2)^3 r, r^2 instead of |r|^2 recomputed, and fused multiply-adds, so each pair
term differs by a few float ulps.  Accelerations are compared against max(||a_ref||, |g| sqrt(n))
because at hydrostatic rest the pressure gradient cancels gravity."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import rel_l2
from gpu_util import dev, host, perturbed

pytestmark = pytest.mark.gpu

TOL_RATE = 5e-5   # rho_dt, vel_dt, dofv (measured <= 1e-5)
TOL_WALL = 2e-6   # wall pressure / density, rhop_sum, w_sum (measured <= 4e-7)


def run_both(oracle, cuda, st, p, wall_rates=False):
    import torch
    from tmp_sph_gb300 import api, solver as S
    P = oracle.params_like(p)
    s = oracle.cell_list(P, st)
    n = len(st["rho"])
    g = {k: dev(s[k], cuda) for k in ("pos", "vel", "rho", "p", "type", "hash", "cell_start",
                                       "cell_end")}
    out = {"rho_dt": torch.zeros(n, device=cuda), "vel_dt": torch.zeros((n, 3), device=cuda),
           "dofv": torch.zeros(n, device=cuda), "rhop_sum": torch.zeros(n, device=cuda),
           "w_sum": torch.zeros(n, device=cuda)}
    with S.Solver(p, n) as sol:
        sol.set_option(api.SPH_OPT_WALL_RATES, int(wall_rates))
        sol.ns(g["pos"], g["vel"], g["rho"], g["p"], g["type"], out["rho_dt"], out["vel_dt"],
               g["cell_start"], g["cell_end"], n, g["hash"], out["dofv"], out["rhop_sum"],
               out["w_sum"])
        flags = sol.error_flags()
    r = oracle.sph_ns(P, s)  # modifies s["p"], s["rho"] of walls in place
    gpu = {k: host(v) for k, v in out.items()}
    gpu["p"] = host(g["p"])
    gpu["rho"] = host(g["rho"])
    return s, r, gpu, flags


def compare(s, r, gpu, report, tag, wall_rates=False):
    fl = s["type"] == 1
    wl = ~fl
    n_f = int(fl.sum())
    e = {
        "rho_dt": rel_l2(gpu["rho_dt"][fl], r["rho_dt"][fl]),
        "vel_dt": rel_l2(gpu["vel_dt"][fl], r["vel_dt"][fl], floor=9.81 * np.sqrt(n_f)),
        "dofv": rel_l2(gpu["dofv"][fl], r["dofv"][fl]),
        "wall_p": rel_l2(gpu["p"][wl], s["p"][wl]),
        "wall_rho": rel_l2(gpu["rho"][wl], s["rho"][wl]),
        "rhop_sum": rel_l2(gpu["rhop_sum"][wl], r["rhop_sum"][wl]),
        "w_sum": rel_l2(gpu["w_sum"][wl], r["w_sum"][wl]),
    }
    for k, v in e.items():
        report(f"{tag} {k}", v, TOL_WALL if k.startswith(("wall", "rhop", "w_")) else TOL_RATE)
    assert e["rho_dt"] < TOL_RATE and e["vel_dt"] < TOL_RATE and e["dofv"] < TOL_RATE, e
    assert e["wall_p"] < TOL_WALL and e["wall_rho"] < TOL_WALL, e
    assert e["rhop_sum"] < TOL_WALL and e["w_sum"] < TOL_WALL, e
    # fluid rows of p / rho are untouched by the neighbour passes
    assert np.array_equal(gpu["p"][fl], s["p"][fl]) and np.array_equal(gpu["rho"][fl], s["rho"][fl])
    if wall_rates:
        n_w = int(wl.sum())
        ew = rel_l2(gpu["vel_dt"][wl], r["vel_dt"][wl], floor=9.81 * np.sqrt(n_w))
        report(f"{tag} wall vel_dt", ew, TOL_RATE)
        assert ew < TOL_RATE
    else:
        assert (gpu["rho_dt"][wl] == 0).all() and (gpu["vel_dt"][wl] == 0).all()


@pytest.mark.parametrize("physics", ["reference", "config"])
@pytest.mark.parametrize("pert", [False, True])
def test_ns_matches_oracle(sphlib, oracle, cuda, report, physics, pert):
    from tmp_sph_gb300 import cases
    st, p = cases.build("small", physics=physics, dx=0.02, jitter=0.01)
    if pert:
        st = perturbed(st)
    s, r, gpu, flags = run_both(oracle, cuda, st, p)
    assert flags == 0
    compare(s, r, gpu, report, f"ns {physics} pert={pert}")


def test_ns_full_small_case(sphlib, oracle, cuda, report):
    """The 133,968-particle dam break at full size, perturbed state."""
    from tmp_sph_gb300 import cases
    st, p = cases.build("small", physics="reference")
    s, r, gpu, _ = run_both(oracle, cuda, perturbed(st), p)
    compare(s, r, gpu, report, "ns small full")


def test_ns_wall_rates_option(sphlib, oracle, cuda, report):
    from tmp_sph_gb300 import cases
    st, p = cases.build("small", physics="reference", dx=0.02)
    s, r, gpu, _ = run_both(oracle, cuda, perturbed(st), p, wall_rates=True)
    compare(s, r, gpu, report, "ns wall rates", wall_rates=True)


def test_ns_two_particles(sphlib, oracle, cuda, report):
    """Hand-built pair: a fluid particle above a wall particle inside the support radius."""
    from tmp_sph_gb300 import cases
    _, p = cases.build("small", physics="reference", dx=0.04)
    st = {"pos": np.array([[0.5, 0.25, 0.30], [0.5, 0.25, 0.30 + 0.8 * p.h]], np.float32),
          "vel": np.array([[0, 0, 0], [0.1, -0.2, 0.3]], np.float32),
          "rho": np.array([1000.0, 1003.0], np.float32),
          "p": np.array([0.0, 1875.0], np.float32), "type": np.array([0, 1], np.int32)}
    s, r, gpu, _ = run_both(oracle, cuda, st, p, wall_rates=True)
    np.testing.assert_allclose(gpu["p"][s["type"] == 0], s["p"][s["type"] == 0], rtol=1e-5)
    np.testing.assert_allclose(gpu["rho_dt"], r["rho_dt"], rtol=1e-4, atol=1e-6)
    np.testing.assert_allclose(gpu["vel_dt"], r["vel_dt"], rtol=1e-4, atol=1e-4)
