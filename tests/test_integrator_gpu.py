"""GPU parity of the drop-in predictor and corrector (src/sph/sph_run.cu:425-519) against the
oracle on identical inputs.  The GPU evaluates rho + rho_dt*dt/2 etc. in float where the
reference promotes to double; results agree to a couple of float ulps."""
from __future__ import annotations

import numpy as np
import pytest

from gpu_util import dev, host, perturbed

pytestmark = pytest.mark.gpu


def test_prediction_and_correction(sphlib, oracle, cuda):
    from tmp_sph_gb300 import cases, solver as S
    st, p = cases.build("small", physics="config", dx=0.02, jitter=0.01)
    st = perturbed(st)
    P = oracle.params_like(p)
    s = oracle.cell_list(P, st)
    n = len(st["rho"])
    rng = np.random.default_rng(5)
    rates = {"rho_dt": rng.normal(0, 50, n).astype(np.float32),
             "vel_dt": rng.normal(0, 5, (n, 3)).astype(np.float32)}
    # one fluid particle outside the escape box
    i_esc = int(np.nonzero(s["type"] == 1)[0][3])
    s["pos"][i_esc, 2] = P.escape_max[2] + 0.01
    tmp = {"pos": np.zeros((n, 3), np.float32), "vel": np.zeros((n, 3), np.float32),
           "rho": np.zeros(n, np.float32)}
    g = {k: dev(s[k], cuda) for k in ("pos", "vel", "rho", "p", "type", "index")}
    gt = {k: dev(v, cuda) for k, v in tmp.items()}
    gr = {k: dev(v, cuda) for k, v in rates.items()}
    S.pc_prediction(p, g["pos"], g["vel"], g["rho"], g["p"], gr["rho_dt"], gr["vel_dt"],
                    g["index"], gt["pos"], gt["vel"], gt["rho"], n, g["type"])
    oracle.pc_prediction(P, s, rates, tmp)
    for k in ("pos", "vel", "rho"):
        np.testing.assert_allclose(host(g[k]), s[k], rtol=2e-6, atol=1e-6, err_msg=k)
    # Tait pressure: float expm1/log1p on the GPU vs double pow in the oracle
    np.testing.assert_allclose(host(g["p"]), s["p"], rtol=1e-5, atol=2e-3, err_msg="p")
    for k in ("pos", "vel", "rho"):
        np.testing.assert_array_equal(host(gt[k]), tmp[k], err_msg="tmp " + k)
    assert np.array_equal(host(g["pos"])[i_esc], np.array(P.escape_park, np.float32))
    # corrector on the predicted state with new rates
    rates2 = {"rho_dt": rng.normal(0, 50, n).astype(np.float32),
              "vel_dt": rng.normal(0, 5, (n, 3)).astype(np.float32)}
    gr2 = {k: dev(v, cuda) for k, v in rates2.items()}
    s2 = {k: host(g[k]).copy() for k in ("pos", "vel", "rho", "p")}
    s2.update(type=s["type"], index=s["index"])
    S.pc_correction(p, g["pos"], g["vel"], g["rho"], g["p"], gr2["rho_dt"], gr2["vel_dt"],
                    g["index"], gt["pos"], gt["vel"], gt["rho"], n, g["type"])
    oracle.pc_correction(P, s2, rates2, tmp)
    for k in ("pos", "vel", "rho"):
        np.testing.assert_allclose(host(g[k]), s2[k], rtol=5e-6, atol=2e-6, err_msg=k)
    np.testing.assert_allclose(host(g["p"]), s2["p"], rtol=2e-5, atol=4e-3, err_msg="p")
    # boundary particles untouched
    wl = s["type"] != 1
    assert np.array_equal(host(g["pos"])[wl], s["pos"][wl])
