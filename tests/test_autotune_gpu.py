"""GPU test of the autotuner: it measures every candidate of its two stages, confirms the model's
best few and the default by running them, picks the fastest measured, and the choice it
returns can be applied and run."""
from __future__ import annotations

import pytest

pytestmark = pytest.mark.gpu


def test_autotune_small_case(sphlib, cuda, report):
    import torch
    from tmp_sph_gb300 import autotune, cases, solver as S
    st, p = cases.build("small", physics="config", dx=0.02)
    best = autotune.tune(p, st, threads=(64, 128), ppt=(1, 2), skins=(0, 100), lanes=(1, 2),
                         divisions=(1, 2), confirm_steps=20)
    # stage 1: 2 x 2 x 2 launch shapes at skin 0.1 kh; stage 2: 2 skins x 2 cell sizes for
    # the best shape, less the one already measured
    assert len(best["table"]) == 8 + 3
    assert all(m["flags"] == 0 for m in best["table"])
    assert all(m["pass_ms_per_half_step"] > 0 and m["rebuild_ms"] > 0 for m in best["table"])
    # skin 0 rebuilds every half step of the profiled steps
    assert all(m["rebuilds_seen"] == 4 for m in best["table"] if m["skin_permille"] == 0)
    assert {m["divisions"] for m in best["table"]} == {1, 2}
    # the choice is the fastest of the confirmation runs, which include the default, unless
    # that one beats the default by less than 1%
    conf = best["confirm"]
    assert any(c["default"] for c in conf) and 2 <= len(conf) <= 4
    fastest = min(c["ms_per_step"] for c in conf)
    base = next(c["ms_per_step"] for c in conf if c["default"])
    assert best["ms_per_step"] == (fastest if fastest <= 0.99 * base else base)
    summ = autotune.summary(best)
    assert summ["ms_per_step"] <= summ["default_ms_per_step"]
    report("autotune small best ms per step", best["ms_per_step"])
    s = torch.cuda.Stream()
    with S.Solver(p, len(st["rho"])) as sol:
        autotune.apply(sol, best)
        sol.upload(st["pos"], st["vel"], st["rho"], st["p"], st["type"], stream=s)
        sol.step(3, stream=s)
        assert sol.error_flags(stream=s) == 0
