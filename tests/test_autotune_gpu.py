"""GPU test of the autotuner: it measures every candidate, picks the cheapest estimate, and
the choice it returns can be applied and run."""
from __future__ import annotations

import pytest

pytestmark = pytest.mark.gpu


def test_autotune_small_case(sphlib, cuda, report):
    import torch
    from tmp_sph_gb300 import autotune, cases, solver as S
    st, p = cases.build("small", physics="config", dx=0.02)
    best = autotune.tune(p, st, threads=(64, 128), ppt=(1, 2), skins=(0, 100), lanes=(1, 2))
    # every combination: 2 x 2 x 2 x 2 candidates
    assert len(best["table"]) == 16
    assert all(m["flags"] == 0 for m in best["table"])
    assert all(m["pass_ms_per_half_step"] > 0 and m["rebuild_ms"] > 0 for m in best["table"])
    # skin 0 rebuilds every half step of the profiled steps
    assert all(m["rebuilds_seen"] == 4 for m in best["table"] if m["skin_permille"] == 0)
    est = min(m["step_ms_estimate"] for m in best["table"])
    assert best["step_ms_estimate"] == est
    report("autotune small best step ms estimate", est)
    s = torch.cuda.Stream()
    with S.Solver(p, len(st["rho"])) as sol:
        autotune.apply(sol, best)
        sol.upload(st["pos"], st["vel"], st["rho"], st["p"], st["type"], stream=s)
        sol.step(3, stream=s)
        assert sol.error_flags(stream=s) == 0
