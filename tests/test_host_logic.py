"""CPU tests of host-side logic: the batch generator, the autotuner's cost model, the launch
count the bench reports, and the study's error metrics."""
from __future__ import annotations

import math

import numpy as np


def test_batch_generator_is_seeded_and_shares_parameters(sphlib):
    from tmp_sph_gb300 import cases
    a, pa = cases.batch(4, dx=0.04, seed=9)
    b, pb = cases.batch(4, dx=0.04, seed=9)
    c, _ = cases.batch(4, dx=0.04, seed=10)
    assert [len(s["rho"]) for s in a] == [len(s["rho"]) for s in b]
    for s, t in zip(a, b):
        assert np.array_equal(s["pos"], t["pos"])
    assert [s["block"] for s in a] != [s["block"] for s in c]
    # one parameter set: c0 from the tallest column, all walls identical
    hmax = max(s["block"][1] for s in a)
    assert math.isclose(pa.cs, 10.0 * math.sqrt(2 * 9.81 * hmax), rel_tol=1e-6)
    nb = {int((s["type"] != 1).sum()) for s in a}
    assert len(nb) == 1
    assert pa.num_particles == sum(len(s["rho"]) for s in a)
    for s in a:
        w, h = s["block"]
        assert 0.2 <= w <= 0.6 and 0.15 <= h <= 0.45


def test_autotune_cost_model():
    from tmp_sph_gb300 import autotune

    class P:
        dt, kh = 1e-4, 0.01

    m0 = {"skin_permille": 0, "pass_ms_per_half_step": 1.0, "rebuild_ms": 3.0}
    m1 = {"skin_permille": 100, "pass_ms_per_half_step": 1.1, "rebuild_ms": 3.5}
    # skin 0 rebuilds every half step: 2 passes + 2 rebuilds
    assert math.isclose(autotune.step_cost(m0, P, 2.0), 2.0 + 6.0)
    # skin 0.1 kh carried at 2 m/s: a rebuild every 0.1*0.01/(2*1e-4) = 5 steps -> 0.2 per step
    assert math.isclose(autotune.step_cost(m1, P, 2.0), 2.2 + 0.2 * 3.5)
    # never more than two rebuilds per step
    assert math.isclose(autotune.step_cost(m1, P, 1e3), 2.2 + 2 * 3.5)
    st = {"type": np.array([1, 1, 0]), "pos": np.array([[0, 0, 0.1], [0, 0, 0.3], [0, 0, 0.9]])}
    assert math.isclose(autotune.surge_speed([st], -9.81), 2 * math.sqrt(9.81 * 0.3))
    # the default the confirmation runs compare against
    assert autotune.default_choice("fp32") == {"threads": 256, "ppt": 1, "lanes": 1,
                                               "skin_permille": 100, "divisions": 3}
    assert autotune.default_choice("mixed")["threads"] == 128
    assert autotune.default_choice("mixed_abs") == autotune.default_choice("fp32")
    # a candidate replaces the default only when it is at least `margin` faster
    runs = [{"ms_per_step": 2.70, "default": True}, {"ms_per_step": 2.69, "default": False}]
    assert autotune.pick(runs, 0.01)["default"]
    runs[1]["ms_per_step"] = 2.60
    assert not autotune.pick(runs, 0.01)["default"]
    assert autotune.pick(runs[:1], 0.01)["default"]


def test_launch_count():
    import importlib.util
    import os
    spec = importlib.util.spec_from_file_location(
        "bench", os.path.join(os.path.dirname(os.path.dirname(__file__)), "bench.py"))
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    # 2^21 cells -> 21-bit keys -> 3 radix passes -> 16 rebuild kernels per rebuild
    assert bench.count_launches(1 << 21, 400, 4, "conditional") == 3 * 400 + 4 * 16
    assert bench.count_launches(1 << 21, 400, 4, "gated") == 400 * (3 + 16)


def test_study_metrics():
    from tmp_sph_gb300 import study
    st = {"type": np.array([1, 1, 0]), "pos": np.zeros((3, 3))}
    a = {"pos": np.array([[1.0, 0, 0], [0, 1, 0], [0, 0, 0]]), "vel": np.ones((3, 3)),
         "rho": np.full(3, 1001.0), "p": np.ones(3)}
    e = study.field_errors(a, a, st)
    assert all(v == 0.0 for v in e.values())
    b = dict(a, rho=np.full(3, 1002.0))
    assert math.isclose(study.field_errors(b, a, st)["drho"], 1.0)
