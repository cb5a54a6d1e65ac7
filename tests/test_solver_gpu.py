"""GPU tests of the resident solver (sph_create / sph_upload / sph_step / sph_download): whole
predictor-corrector steps against the oracle's reference step loop
(src/sph/sph_run.cu:285-336), CUDA-graph replay against plain launches, the end-to-end host
call, and full-size properties of the 4.96M-particle case.

The resident solver keeps particles in cell order between steps, so particles that share a
cell are summed in a different order than the reference (which returns to original order
every half step); the fields therefore agree to FP32 rounding growth, not bit for bit."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


def run_gpu(st, p, nsteps, graph=True, stream=None, precision="fp32"):
    import torch
    from tmp_sph_gb300 import api, solver as S
    n = len(st["rho"])
    s = stream or torch.cuda.Stream()
    with S.Solver(p, n, precision=precision) as sol:
        sol.set_option(api.SPH_OPT_USE_GRAPH, int(graph))
        with torch.cuda.stream(s):
            sol.upload(st["pos"], st["vel"], st["rho"], st["p"], st["type"], stream=s)
            sol.step(nsteps, stream=s)
            out = sol.download(stream=s)
        flags = sol.error_flags(stream=s)
        assert sol.steps_taken() == nsteps
    return out, flags


def field_errors(out, ref, st):
    fl = st["type"] == 1
    n_f = int(fl.sum())
    return {
        "disp": rel_l2(out["pos"][fl] - st["pos"][fl], ref["pos"][fl] - st["pos"][fl]),
        "vel": rel_l2(out["vel"][fl], ref["vel"][fl], floor=1e-3 * np.sqrt(n_f)),
        "drho": rel_l2(out["rho"][fl] - 1000.0, ref["rho"][fl] - 1000.0),
        "p": rel_l2(out["p"][fl], ref["p"][fl]),
    }


@pytest.mark.parametrize("physics", ["reference", "config"])
def test_steps_match_oracle(sphlib, oracle, cuda, report, physics):
    from tmp_sph_gb300 import cases
    st, p = cases.build("small", physics=physics, dx=0.02, jitter=0.01)
    P = oracle.params_like(p)
    # After one step the displacement (~3.5e-7 m) is only ~50 ulp of the position, so a
    # velocity that differs in its last bits flips the rounding of pos + dt v for a few
    # particles: 1-ulp flips with probability ~1e-4 per coordinate give disp errors of ~1e-4.
    # The positions themselves are checked to within 1 ulp.
    for nsteps, tol, tol_disp in ((1, 2e-5, 5e-4), (20, 2e-4, 2e-4)):  # measured 2e-6 / 2e-5
        out, flags = run_gpu(st, p, nsteps)
        ref = oracle.run(P, st, nsteps)
        assert flags == 0
        e = field_errors(out, ref, st)
        for k, v in e.items():
            report(f"solver {physics} {nsteps} steps {k}", v, tol_disp if k == "disp" else tol)
        assert e["disp"] < tol_disp and all(v < tol for k, v in e.items() if k != "disp"), \
            (nsteps, e)
        if nsteps == 1:
            ulp = np.spacing(np.abs(ref["pos"]).astype(np.float32))
            dist = np.abs(out["pos"] - ref["pos"]) / ulp
            w = np.unravel_index(np.argmax(dist), dist.shape)
            report(f"solver {physics} 1 step max position difference in ulp", dist.max(), 2.0)
            assert dist.max() <= 2.0, (w, out["pos"][w[0]], ref["pos"][w[0]], st["pos"][w[0]],
                                       out["vel"][w[0]], ref["vel"][w[0]], st["type"][w[0]])
        wl = st["type"] != 1
        assert np.array_equal(out["pos"][wl], st["pos"][wl])
        assert np.array_equal(out["type"], st["type"])
        np.testing.assert_allclose(out["p"][wl], ref["p"][wl], rtol=1e-3, atol=1.0)


def test_graph_replay_is_bitwise_identical(sphlib, cuda):
    """Graph replay (rebuild kernels under conditional nodes, or gated) and plain launches give
    the same bits, with list rebuilds forced by fast flow as well as skipped."""
    from tmp_sph_gb300 import api, cases
    from gpu_util import perturbed
    st, p = cases.build("small", physics="config", dx=0.02, jitter=0.01)
    for s in (st, perturbed(st, vamp=2.0, ramp=0.0)):
        a, _ = run_gpu(s, p, 7, graph=True)
        b, _ = run_gpu(s, p, 7, graph=False)
        c, _ = run_opts(s, p, 7, {api.SPH_OPT_CONDITIONAL_GRAPH: 0})
        for k in ("pos", "vel", "rho", "p", "type"):
            assert np.array_equal(a[k], b[k]), k
            assert np.array_equal(a[k], c[k]), k


def run_opts(st, p, nsteps, opts):
    import torch
    from tmp_sph_gb300 import solver as S
    n = len(st["rho"])
    s = torch.cuda.Stream()
    with S.Solver(p, n) as sol:
        for k, v in opts.items():
            sol.set_option(k, v)
        sol.upload(st["pos"], st["vel"], st["rho"], st["p"], st["type"], stream=s)
        sol.step(nsteps, stream=s)
        out = sol.download(stream=s)
        out["rebuilds"] = sol.rebuild_count(stream=s)
        flags = sol.error_flags(stream=s)
    return out, flags


def test_neighbor_list_matches_cell_walk(sphlib, cuda):
    """Without a skin the list is rebuilt every half step and the one-lane list passes visit
    the same pairs in the same order as passes that walk the cells themselves: bit-identical
    steps."""
    from tmp_sph_gb300 import api, cases
    st, p = cases.build("small", physics="config", dx=0.02, jitter=0.01)
    a, fa = run_opts(st, p, 5, {api.SPH_OPT_SKIN_PERMILLE: 0, api.SPH_OPT_NEIGHBOR_LIST: 1,
                                api.SPH_OPT_LANES_PER_PARTICLE: 1})
    b, fb = run_opts(st, p, 5, {api.SPH_OPT_SKIN_PERMILLE: 0, api.SPH_OPT_NEIGHBOR_LIST: 0})
    assert fa == 0 and fb == 0
    for k in ("pos", "vel", "rho", "p"):
        assert np.array_equal(a[k], b[k]), k


def test_neighbor_list_overflow_falls_back(sphlib, cuda):
    """With a 16-slot list every fluid particle overflows: it is flagged and walks its cells,
    giving the same result as the one-lane list passes."""
    from tmp_sph_gb300 import api, cases
    st, p = cases.build("small", physics="config", dx=0.02, jitter=0.01)
    one = {api.SPH_OPT_LANES_PER_PARTICLE: 1}
    for skin in (0, 100):
        a, fa = run_opts(st, p, 3, {**one, api.SPH_OPT_SKIN_PERMILLE: skin,
                                    api.SPH_OPT_NEIGHBOR_CAP: 8})
        b, fb = run_opts(st, p, 3, {**one, api.SPH_OPT_SKIN_PERMILLE: skin})
        assert fa & api.SPH_FLAG_NEIGHBOR_OVERFLOW and fb == 0
        for k in ("pos", "vel", "rho", "p"):
            assert np.array_equal(a[k], b[k]), (skin, k)


@pytest.mark.parametrize("skin", [100, 300])
def test_skin_reuse_matches_oracle(sphlib, oracle, cuda, report, skin):
    """Reusing the cell and neighbour lists while particles stay within skin/2 evaluates the
    same pairs (r < kh) as rebuilding every half step: 20 steps agree with the oracle within
    float rounding, and the lists were rebuilt fewer times than there were half steps."""
    import torch
    from tmp_sph_gb300 import api, cases, solver as S
    st, p = cases.build("small", physics="config", dx=0.02, jitter=0.01)
    n = len(st["rho"])
    s = torch.cuda.Stream()
    with S.Solver(p, n) as sol:
        sol.set_option(api.SPH_OPT_SKIN_PERMILLE, skin)
        sol.upload(st["pos"], st["vel"], st["rho"], st["p"], st["type"], stream=s)
        sol.step(20, stream=s)
        out = sol.download(stream=s)
        rebuilds = sol.rebuild_count(stream=s)
        flags = sol.error_flags(stream=s)
    ref = oracle.run(oracle.params_like(p), st, 20)
    e = field_errors(out, ref, st)
    for k, v in e.items():
        report(f"skin {skin} 20 steps {k}", v, 2e-4)
    report(f"skin {skin} rebuilds in 40 half steps", rebuilds)
    assert flags == 0
    assert all(v < 2e-4 for v in e.values()), e
    assert 1 <= rebuilds < 40


def test_grid_change_mid_run_matches_oracle(sphlib, oracle, cuda, report):
    """Changing the skin (and so the cell grid) or re-setting the parameters between steps
    recomputes the cell keys of the resident particles before the next rebuild: the run still
    matches the oracle."""
    import torch
    from tmp_sph_gb300 import api, cases, solver as S
    st, p = cases.build("small", physics="config", dx=0.02, jitter=0.01)
    n = len(st["rho"])
    s = torch.cuda.Stream()
    with S.Solver(p, n) as sol:
        sol.set_option(api.SPH_OPT_SKIN_PERMILLE, 100)
        sol.upload(st["pos"], st["vel"], st["rho"], st["p"], st["type"], stream=s)
        sol.step(3, stream=s)
        sol.set_option(api.SPH_OPT_SKIN_PERMILLE, 0)
        sol.step(3, stream=s)
        sol.set_option(api.SPH_OPT_SKIN_PERMILLE, 300)
        sol.step(2, stream=s)
        sol.set_params(p)
        sol.step(2, stream=s)
        out = sol.download(stream=s)
        flags = sol.error_flags(stream=s)
    ref = oracle.run(oracle.params_like(p), st, 10)
    e = field_errors(out, ref, st)
    for k, v in e.items():
        report(f"grid change mid run 10 steps {k}", v, 2e-4)
    assert flags == 0
    assert all(v < 2e-4 for v in e.values()), e


def test_skin_reuse_fast_flow(sphlib, oracle, cuda, report):
    """Fast random velocities (±2 m/s) force frequent rebuilds; results still match."""
    from tmp_sph_gb300 import api, cases
    from gpu_util import perturbed
    st, p = cases.build("small", physics="config", dx=0.02, jitter=0.01)
    st = perturbed(st, vamp=2.0, ramp=0.0)
    out, flags = run_opts(st, p, 6, {api.SPH_OPT_SKIN_PERMILLE: 100})
    ref = oracle.run(oracle.params_like(p), st, 6)
    e = field_errors(out, ref, st)
    for k, v in e.items():
        report(f"skin fast flow 6 steps {k}", v, 2e-4)
    report("skin fast flow rebuilds in 12 half steps", out["rebuilds"])
    assert flags == 0
    assert all(v < 2e-4 for v in e.values()), e
    assert out["rebuilds"] >= 2


def test_upload_download_roundtrip(sphlib, cuda):
    from tmp_sph_gb300 import cases
    st, p = cases.build("small", physics="config", dx=0.02, jitter=0.01)
    out, flags = run_gpu(st, p, 0)
    for k in ("pos", "vel", "rho", "p", "type"):
        assert np.array_equal(out[k], st[k]), k


def test_download_into_device_memory(sphlib, cuda):
    """sph_download with to_host = 0 writes the same state, in original order, into device
    arrays as the host download; a NULL array is skipped."""
    import torch
    from tmp_sph_gb300 import cases, solver as S
    st, p = cases.build("small", physics="config", dx=0.02, jitter=0.01)
    n = len(st["rho"])
    s = torch.cuda.Stream()
    with S.Solver(p, n) as sol:
        sol.upload(st["pos"], st["vel"], st["rho"], st["p"], st["type"], stream=s)
        sol.step(2, stream=s)
        host = sol.download(stream=s)
        dev = {"pos": torch.full((n, 3), -1.0, device=cuda),
               "vel": torch.full((n, 3), -1.0, device=cuda),
               "rho": torch.full((n,), -1.0, device=cuda),
               "type": torch.full((n,), -7, dtype=torch.int32, device=cuda)}
        torch.cuda.synchronize()  # the fills above ran on torch's stream, the download runs on s
        sol.download_device(dev, stream=s)
        s.synchronize()
        assert sol.error_flags(stream=s) == 0
    for k in ("pos", "vel", "rho", "type"):
        assert np.array_equal(dev[k].cpu().numpy(), host[k]), k


def test_step_host_matches_device_path(sphlib, cuda):
    import torch
    from tmp_sph_gb300 import cases, solver as S
    st, p = cases.build("small", physics="config", dx=0.02, jitter=0.01)
    dev_out, _ = run_gpu(st, p, 3, graph=False)
    n = len(st["rho"])
    hst = {k: torch.from_numpy(np.ascontiguousarray(st[k])).pin_memory().numpy()
           for k in ("pos", "vel", "rho", "p", "type")}
    s = torch.cuda.Stream()
    with S.Solver(p, n) as sol:
        sol.set_option(1, 0)
        sol.step_host(hst, 3, stream=s)
    for k in ("pos", "vel", "rho", "p"):
        assert np.array_equal(hst[k], dev_out[k]), k


def test_escape_and_out_of_grid_flags(sphlib, cuda):
    """A fluid particle above the escape box is parked (src/sph/sph_run.cu:437-447); one
    outside the grid is clamped into it and raises SPH_FLAG_OUT_OF_GRID, without a fault."""
    from tmp_sph_gb300 import api, cases
    st, p = cases.build("small", physics="config", dx=0.04)
    fl = np.nonzero(st["type"] == 1)[0]
    st["pos"][fl[0]] = (0.5, 0.25, p.escape_max[2] + 0.02)
    out, flags = run_gpu(st, p, 1)
    assert np.array_equal(out["pos"][fl[0]], np.array(p.escape_park, np.float32))
    assert flags == 0
    st["pos"][fl[1]] = (0.5, 0.25, p.grid_max[2] + 1.0)
    out, flags = run_gpu(st, p, 1)
    assert flags & api.SPH_FLAG_OUT_OF_GRID
    assert np.array_equal(out["pos"][fl[1]], np.array(p.escape_park, np.float32))


def test_api_errors(sphlib, cuda):
    import ctypes as C
    from tmp_sph_gb300 import api, cases
    _, p = cases.build("small", physics="config", dx=0.04)
    L = api.lib()
    h = C.c_void_p()
    assert L.sph_create(C.byref(p), p.num_particles, C.byref(h)) == api.SPH_OK
    try:
        assert L.sph_step(h, 1, None) == api.SPH_ERR_STATE
        assert L.sph_upload(h, None, None, None, None, None, p.num_particles + 1, 1, None) == api.SPH_ERR_ARG
        assert L.sph_ctx_set_option(h, 99, 1) == api.SPH_ERR_ARG
        bad = api.SphParams.from_buffer_copy(p)
        bad.cell_size = bad.kh * 0.5
        assert L.sph_set_params(h, C.byref(bad)) == api.SPH_ERR_ARG
    finally:
        L.sph_destroy(h)


def test_profile_phases(sphlib, cuda):
    import torch
    from tmp_sph_gb300 import api, cases, solver as S
    st, p = cases.build("small", physics="config", dx=0.02)
    n = len(st["rho"])
    s = torch.cuda.Stream()
    with S.Solver(p, n) as sol:
        sol.set_option(api.SPH_OPT_PROFILE, 1)
        sol.upload(st["pos"], st["vel"], st["rho"], st["p"], st["type"], stream=s)
        sol.step(3, stream=s)
        prof = sol.profile()
    assert set(prof) == set(api.PHASE_NAMES)
    assert all(v["launches"] == 6 and v["ms"] > 0 for v in prof.values())


def test_large_case_properties(sphlib, cuda, report):
    """The 4,963,548-particle case (dx 2.5 mm, jitter 0.01 dx): five steps stay finite and
    physical, walls stay put, the particle ids stay a permutation, the sorted cell keys are
    sorted and the dense cell starts bracket them."""
    import torch
    from tmp_sph_gb300 import api, cases, solver as S
    st, p = cases.build("large", physics="config")
    n = len(st["rho"])
    assert n == 4963548
    s = torch.cuda.Stream()
    with S.Solver(p, n) as sol:
        sol.upload(st["pos"], st["vel"], st["rho"], st["p"], st["type"], stream=s)
        sol.step(5, stream=s)
        out = sol.download(stream=s)
        cs_ptr, id_ptr, key_ptr, ncells = sol.sorted_view()
        import ctypes as C
        keys = np.zeros(n, np.int32)
        ids = np.zeros(n, np.int32)
        cs = np.zeros(ncells + 1, np.int32)
        torch.cuda.synchronize()
        rt = C.CDLL("libcudart.so.13")  # already loaded as the library's dependency
        rt.cudaMemcpy.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int]
        assert rt.cudaMemcpy(keys.ctypes.data, key_ptr, n * 4, 2) == 0
        assert rt.cudaMemcpy(ids.ctypes.data, id_ptr, n * 4, 2) == 0
        assert rt.cudaMemcpy(cs.ctypes.data, cs_ptr, (ncells + 1) * 4, 2) == 0
        flags = sol.error_flags(stream=s)
    assert flags == 0
    fl = st["type"] == 1
    for k in ("pos", "vel", "rho", "p"):
        assert np.isfinite(out[k]).all(), k
    assert np.array_equal(out["pos"][~fl], st["pos"][~fl])
    assert np.abs(out["vel"][fl]).max() < 1.0
    assert (out["rho"][fl] >= 1000.0).all() and (out["rho"][fl] < 1050.0).all()
    assert np.array_equal(np.sort(ids), np.arange(n))
    assert (np.diff(keys) >= 0).all()
    assert cs[0] == 0 and cs[-1] == n and (np.diff(cs) >= 0).all()
    occ = np.unique(keys)
    assert (cs[occ + 1] - cs[occ] == np.bincount(keys, minlength=ncells)[occ]).all()
    report("large 5 steps max |v|", float(np.abs(out["vel"][fl]).max()))


@pytest.mark.parametrize("threads,ppt", [(64, 1), (256, 1), (128, 2), (96, 4)])
def test_launch_shape_is_bitwise_neutral(sphlib, cuda, threads, ppt):
    """Threads per block and particles per thread of the neighbour kernels change only the
    launch shape: each particle's arithmetic and order are the same, so are the bits."""
    from tmp_sph_gb300 import api, cases
    from gpu_util import perturbed
    st, p = cases.build("small", physics="config", dx=0.02, jitter=0.01)
    st = perturbed(st, vamp=2.0, ramp=0.0)
    a, fa = run_opts(st, p, 6, {})
    b, fb = run_opts(st, p, 6, {api.SPH_OPT_BLOCK_THREADS: threads,
                                api.SPH_OPT_PARTICLES_PER_THREAD: ppt})
    assert fa == 0 and fb == 0 and a["rebuilds"] == b["rebuilds"]
    for k in ("pos", "vel", "rho", "p", "type"):
        assert np.array_equal(a[k], b[k]), k


def test_launch_shape_options_are_checked(sphlib):
    from tmp_sph_gb300 import api, cases, solver as S
    st, p = cases.build("small", physics="config", dx=0.04)
    with S.Solver(p, len(st["rho"])) as sol:
        lib = api.lib()
        for bad in (-32, 16, 48, 288):
            assert lib.sph_ctx_set_option(sol.handle, api.SPH_OPT_BLOCK_THREADS, bad) == \
                api.SPH_ERR_ARG
        # 0 restores the precision's default: 256 threads in FP32
        assert lib.sph_ctx_set_option(sol.handle, api.SPH_OPT_BLOCK_THREADS, 0) == api.SPH_OK
        assert sol.get_option(api.SPH_OPT_BLOCK_THREADS) == 256
        for bad in (0, 65):
            assert lib.sph_ctx_set_option(sol.handle, api.SPH_OPT_PARTICLES_PER_THREAD, bad) == \
                api.SPH_ERR_ARG
        assert lib.sph_ctx_set_option(sol.handle, api.SPH_OPT_BLOCK_THREADS, 192) == api.SPH_OK


def test_obstacle_case_matches_oracle(sphlib, oracle, cuda, report):
    """The obstacle geometry (rigid box particles, kind 2, act as boundary particles as in the
    reference): 10 resident steps against the oracle at dx = 3 cm (66,279 particles), in FP32
    and in mixed precision on FP32 positions."""
    import torch
    from tmp_sph_gb300 import cases, solver as S
    st, p = cases.build("obstacle", physics="config", dx=0.03)
    assert (st["type"] == 2).sum() > 0
    rig = st["type"] == 2
    out, flags = run_gpu(st, p, 10)
    ref = oracle.run(oracle.params_like(p), st, 10)
    assert flags == 0
    e = field_errors(out, ref, st)
    for k, v in e.items():
        report(f"obstacle fp32 10 steps {k}", v, 2e-4)
    assert all(v < 2e-4 for v in e.values()), e
    assert np.array_equal(out["pos"][rig], st["pos"][rig])
    # mixed precision on FP32 positions integrates in FP64: against the FP64 oracle, in full
    # precision (a displacement of 10 steps from rest is below the float spacing of positions)
    s = torch.cuda.Stream()
    with S.Solver(p, len(st["rho"]), precision="mixed_abs") as sol:
        sol.upload(st["pos"], st["vel"], st["rho"], st["p"], st["type"], stream=s)
        sol.step(10, stream=s)
        outd = sol.download_f64(stream=s)
        assert sol.error_flags(stream=s) == 0
    refd = oracle.run(oracle.params_like(p), st, 10, dtype=np.float64)
    fl = st["type"] == 1
    x0 = st["pos"][fl].astype(np.float64)
    ed = {"disp": rel_l2(outd["pos"][fl] - x0, refd["pos"][fl] - x0),
          "vel": rel_l2(outd["vel"][fl], refd["vel"][fl], floor=1e-3 * np.sqrt(fl.sum())),
          "drho": rel_l2(outd["rho"][fl] - 1000.0, refd["rho"][fl] - 1000.0)}
    for k, v in ed.items():
        report(f"obstacle mixed_abs vs fp64 oracle 10 steps {k}", v, 1e-4)
    assert all(v < 1e-4 for v in ed.values()), ed
    assert np.array_equal(outd["pos"][rig], st["pos"][rig].astype(np.float64))


def test_rebuild_test_follows_relative_motion(sphlib, oracle, cuda, report):
    """The lists are rebuilt when the box of all displacements since the last build has a
    half-diagonal beyond skin/2: a block carried at 1 m/s past static walls keeps them for
    about skin/v (twice as long as a test on the largest displacement would), the results match
    the oracle, and with every list overflowed (cell walks from the cells of the last build)
    they are the same bits."""
    from tmp_sph_gb300 import api, cases
    st, p = cases.build("small", physics="config", dx=0.02, jitter=0.01)
    fl = st["type"] == 1
    st["vel"][fl] = np.array([1.0, 0.0, 0.0], np.float32)
    steps = 60
    fixed = {api.SPH_OPT_SKIN_PERMILLE: 100, api.SPH_OPT_ADAPTIVE_SKIN: 0,
             api.SPH_OPT_LANES_PER_PARTICLE: 1}  # list passes in walk order
    out, flags = run_opts(st, p, steps, fixed)
    skin = 0.1 * float(p.kh)
    per_build = skin / (1.0 * float(p.dt))  # steps a uniform 1 m/s carry takes to reach skin
    report("uniform carry: list rebuilds in 60 steps", out["rebuilds"], 1 + steps / per_build)
    assert flags == 0
    assert out["rebuilds"] <= 2 + steps / per_build
    ref = oracle.run(oracle.params_like(p), st, steps)
    e = field_errors(out, ref, st)
    for k, v in e.items():
        report(f"uniform carry 60 steps {k}", v, 2e-4)
    assert all(v < 2e-4 for v in e.values()), e
    walk, wflags = run_opts(st, p, steps, {**fixed, api.SPH_OPT_NEIGHBOR_CAP: 8})
    assert wflags & api.SPH_FLAG_NEIGHBOR_OVERFLOW
    assert walk["rebuilds"] == out["rebuilds"]
    for k in ("pos", "vel", "rho", "p"):
        assert np.array_equal(walk[k], out[k]), k


def test_adaptive_skin(sphlib, oracle, cuda, report):
    """The lists start tight (skin 0.02 kh) and stay near that while the flow is slow; fast flow
    widens them towards the skin option; with the option off they use it throughout.  The
    fields match the oracle either way."""
    import torch
    from tmp_sph_gb300 import api, cases, solver as S
    from gpu_util import perturbed
    st, p = cases.build("small", physics="config", dx=0.02, jitter=0.01)
    P = oracle.params_like(p)
    for name, state, steps in (("rest", st, 20), ("fast", perturbed(st, vamp=2.0, ramp=0.0), 30)):
        s = torch.cuda.Stream()
        with S.Solver(p, len(state["rho"])) as sol:
            sol.set_option(api.SPH_OPT_SKIN_PERMILLE, 100)
            sol.upload(state["pos"], state["vel"], state["rho"], state["p"], state["type"],
                       stream=s)
            assert abs(sol.list_skin(stream=s) - 0.02) < 1e-6
            sol.step(steps, stream=s)
            skin = sol.list_skin(stream=s)
            rebuilds = sol.rebuild_count(stream=s)
            out = sol.download(stream=s)
            assert sol.error_flags(stream=s) == 0
            sol.set_option(api.SPH_OPT_ADAPTIVE_SKIN, 0)
            assert abs(sol.list_skin(stream=s) - 0.1) < 1e-6
        report(f"adaptive skin, {name}: skin after {steps} steps", skin)
        report(f"adaptive skin, {name}: rebuilds", rebuilds)
        if name == "rest":
            assert 0.02 - 1e-6 <= skin <= 0.03
        else:
            assert skin > 0.04 and rebuilds >= 3
        ref = oracle.run(P, state, steps)
        e = field_errors(out, ref, state)
        for k, v in e.items():
            report(f"adaptive skin, {name}, {steps} steps {k}", v, 2e-4)
        assert all(v < 2e-4 for v in e.values()), (name, e)
