"""GPU tests of the asynchronous snapshot (sph_snapshot_begin / wait) and the frame writer:
a snapshot holds the state of the moment it was begun although steps run while it is copied,
and the VTK frames hold the states of their steps."""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_snapshot_overlaps_steps(sphlib, cuda):
    import torch
    from tmp_sph_gb300 import api, cases, solver as S
    from gpu_util import perturbed
    st, p = cases.build("small", physics="config", dx=0.02)
    st = perturbed(st, vamp=1.0, ramp=0.0)
    n = len(st["rho"])
    s = torch.cuda.Stream()
    host = {"pos": torch.empty((n, 3)).pin_memory(), "vel": torch.empty((n, 3)).pin_memory(),
            "rho": torch.empty(n).pin_memory(), "p": torch.empty(n).pin_memory(),
            "type": torch.empty(n, dtype=torch.int32).pin_memory()}
    with S.Solver(p, n) as sol:
        sol.upload(st["pos"], st["vel"], st["rho"], st["p"], st["type"], stream=s)
        sol.step(3, stream=s)
        ref = sol.download(stream=s)
        lib = api.lib()
        assert lib.sph_snapshot_begin(sol.handle, host["pos"].data_ptr(), host["vel"].data_ptr(),
                                      host["rho"].data_ptr(), host["p"].data_ptr(),
                                      host["type"].data_ptr(), s.cuda_stream) == 0
        sol.step(5, stream=s)  # runs while the snapshot is copied
        done = ctypes.c_int(-1)
        assert lib.sph_snapshot_query(sol.handle, ctypes.byref(done)) == 0 and done.value in (0, 1)
        assert lib.sph_snapshot_wait(sol.handle) == 0
        after = sol.download(stream=s)
    for k in ("pos", "vel", "rho", "p", "type"):
        assert np.array_equal(host[k].numpy(), ref[k]), k
    assert not np.array_equal(after["pos"], ref["pos"])


def test_frame_writer(sphlib, cuda, tmp_path):
    import torch
    from tmp_sph_gb300 import cases, output, solver as S
    st, p = cases.build("small", physics="config", dx=0.02)
    n = len(st["rho"])
    s = torch.cuda.Stream()
    refs = {}
    with S.Solver(p, n) as sol:
        sol.upload(st["pos"], st["vel"], st["rho"], st["p"], st["type"], stream=s)
        with output.FrameWriter(sol, str(tmp_path)) as fw:
            for i in range(4):
                sol.step(2, stream=s)
                fw.frame(2 * (i + 1), stream=s)
                refs[2 * (i + 1)] = sol.download(stream=s)
    for step, ref in refs.items():
        got = output.read_vtk(str(tmp_path / f"fluid_t={step}.vtk"))
        for k in ("pos", "vel", "p", "type"):
            assert np.array_equal(got[k], ref[k]), (step, k)
