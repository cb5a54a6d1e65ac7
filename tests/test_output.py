"""The legacy-VTK writer (sph_write_vtk) on the CPU: binary big-endian and text files read
back equal to what was written, in the reference's layout (src/io/io.cu:154-199,
opt_src_v3/io/io.cu:121-200)."""
from __future__ import annotations

import numpy as np
import pytest


@pytest.mark.parametrize("binary", [True, False])
def test_vtk_round_trip(sphlib, tmp_path, binary):
    from tmp_sph_gb300 import output
    rng = np.random.default_rng(4)
    n = 1000
    pos = rng.uniform(-1, 1, (n, 3)).astype(np.float32)
    vel = rng.normal(size=(n, 3)).astype(np.float32)
    p = rng.uniform(0, 5e3, n).astype(np.float32)
    t = rng.integers(0, 3, n).astype(np.int32)
    path = str(tmp_path / "f.vtk")
    output.write_vtk(path, pos, vel, p, t, binary=binary)
    head = open(path, "rb").read(120).split(b"\n")
    assert head[0] == b"# vtk DataFile Version 3.0"
    assert head[2] == (b"BINARY" if binary else b"ASCII")
    assert head[3] == b"DATASET UNSTRUCTURED_GRID" and head[4] == b"POINTS 1000 float"
    back = output.read_vtk(path)
    for k, v in (("pos", pos), ("vel", vel), ("p", p), ("type", t)):
        assert np.array_equal(back[k], v), k


def test_vtk_arguments(sphlib, tmp_path):
    from tmp_sph_gb300 import api
    lib = api.lib()
    assert lib.sph_write_vtk(None, 1, None, None, None, None, 1) == api.SPH_ERR_ARG
    assert lib.sph_write_vtk(str(tmp_path / "e.vtk").encode(), 0, None, None, None, None, 1) == 0
    assert lib.sph_write_vtk(str(tmp_path / "x.vtk").encode(), 5, None, None, None, None, 1) == \
        api.SPH_ERR_ARG
    assert lib.sph_write_vtk(b"/nonexistent-dir/x.vtk", 0, None, None, None, None, 1) == \
        api.SPH_ERR_ARG
