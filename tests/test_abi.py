"""CPU tests of the C-ABI library: it loads without a GPU, exports every function declared in
include/sph_gb300.h and the reference-signature shim, and its host-side logic (parameter
derivation, initial conditions, the reference's text input format) is right.  No kernel is
launched here."""
from __future__ import annotations

import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "sph_gb300.h")


def header_functions() -> list[str]:
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"^[A-Za-z_][\w\s\*]*?\b(sph_\w+)\s*\(", src, flags=re.M)))


def test_header_lists_functions():
    fns = header_functions()
    assert "sph_calc_hash" in fns and "sph_step" in fns and len(fns) >= 30


def test_library_exports_every_header_function(sphlib):
    from tmp_sph_gb300 import api
    fns = header_functions()
    missing = [f for f in fns if not hasattr(sphlib, f)]
    assert not missing, missing
    # the binding describes every exported function and nothing else
    assert sorted(api.EXPORTED) == fns


def test_reference_signature_shim_exported(sphlib):
    from tmp_sph_gb300 import api
    out = subprocess.run(["nm", "-D", "--defined-only", "-C", api.LIB_PATH], capture_output=True,
                         text=True, check=True).stdout
    expected = [
        "calcHash(float*, int*, int*, int)",
        "sortParticles(int*, int*, int)",
        "reorder(float*, float*, float*, float*, int*, int*, float*, float*, float*, float*, "
        "int*, int*, int*, int*, int*, int*, int, SimParams*)",
        "recover(float*, float*, float*, float*, int, int*, int*, int*, float*, float*, float*, "
        "float*, int*, int*)",
        "SPH_NS_simpleversion(float*, float*, float*, float*, int*, float*, float*, int*, int*, "
        "int, int*, int, float*, float*, float*)",
        "PC_prediction(float*, float*, float*, float*, float*, float*, int*, int*, float*, "
        "float*, float*, int, int*)",
        "PC_correction(float*, float*, float*, float*, float*, float*, int*, int*, float*, "
        "float*, float*, int, int*)",
        "iDivUp(int, int)",
        "computeGridSize(int, int, int&, int&)",
    ]
    for sig in expected:
        assert sig in out, sig


def test_status_strings(sphlib):
    from tmp_sph_gb300 import api
    assert api.status_string(api.SPH_OK) == "ok"
    assert "scratch" in api.status_string(api.SPH_ERR_SCRATCH)
    assert b"sm_103a" in sphlib.sph_version()


def test_reference_params_match_oracle(sphlib, oracle):
    """The reference host block (src/sph/sph_run.cu:60-101) derived by the library and by the
    oracle gives identical bits for every field."""
    from tmp_sph_gb300 import api
    for dx, dims in [(0.01, (3.221, 1.0, 1.0)), (0.005, (1.0, 0.5, 0.6)), (0.0025, (1.0, 0.5, 0.6))]:
        a = api.params_reference(dx, *dims, 1000, 10).as_dict()
        b = oracle.params_reference(dx, *dims, 1000, 10).as_dict()
        assert a == b
    p = api.params_reference(0.01, 3.221, 1.0, 1.0)
    # spot values of the reference case
    assert p.grid_dim[0] == 115 and p.num_cells == p.grid_dim[0] * p.grid_dim[1] * p.grid_dim[2]
    assert p.h == np.float32(0.015) and p.kh == np.float32(0.03) and p.cell_size == p.kh


def test_config_params_match_oracle(sphlib, oracle):
    from tmp_sph_gb300 import api, cases
    for name in ("small", "large", "precision", "obstacle"):
        d = cases.geometry(name)
        c = cases.config(d, "config", 100, 10)
        a = api.params_derive(c).as_dict()
        b = oracle.params_general(c.dx, c.h_factor, c.rho0, c.cs, c.gravity, c.delta, c.alpha,
                                  c.dt, c.cfl, c.eos, c.tait_gamma, list(c.domain_min),
                                  list(c.domain_max), c.pad, c.cell_factor, 100, 10).as_dict()
        for k in ("dt", "cell_size", "grid_min", "grid_max", "grid_dim", "num_cells", "h", "kh",
                  "eta", "adh", "mass", "tait_b"):
            assert a[k] == b[k], (name, k, a[k], b[k])


def test_params_reference_roundtrip(sphlib):
    from tmp_sph_gb300 import api
    p = api.params_reference(0.01, 3.221, 1.0, 1.0, 1140638, 470903)
    r = api.params_to_reference(p)
    assert r.hash_max == r.gridxdim * r.gridydim * r.gridzdim + r.gridxdim * r.gridydim + r.gridxdim
    q = api.params_from_reference(r)
    for k in ("cell_size", "grid_min", "grid_dim", "num_cells", "h", "kh", "adh", "mass", "dt"):
        assert getattr(q, k) == getattr(p, k) if not hasattr(getattr(q, k), "__len__") else \
            list(getattr(q, k)) == list(getattr(p, k))


def test_params_reject_bad_config(sphlib):
    from tmp_sph_gb300 import api, cases
    c = cases.config(cases.geometry("small"))
    c.dx = 0.0
    with pytest.raises(api.SphError):
        api.params_derive(c)


@pytest.mark.parametrize("name,nf,nb", [("small", 60000, 73968), ("large", 3840000, 1123548),
                                        ("precision", 480000, 285828),
                                        ("obstacle", 5280000, 1503620)])
def test_dam_break_counts(sphlib, name, nf, nb):
    """Counts of the benchmark geometries: fluid on the lattice, three wall layers outside the
    floor and the four side walls, plus the rigid obstacle box (81,920 at dx 0.005)."""
    from tmp_sph_gb300 import api, cases
    assert api.dam_break_count(cases.geometry(name)) == (nf, nb)


def test_dam_break_generate(sphlib):
    from tmp_sph_gb300 import api, cases
    st = api.dam_break_generate(cases.geometry("small", dx=0.02))
    t = st["type"]
    nb = st["n_boundary"]
    assert (t[:nb] != 1).all() and (t[nb:] == 1).all()
    fl = st["pos"][nb:]
    assert fl.min() > 0 and fl[:, 0].max() < 0.4 and fl[:, 2].max() < 0.3
    # hydrostatic: deepest fluid has the largest pressure, rho >= rho0
    assert st["p"][nb:].max() > 0.9 * 1000 * 9.81 * 0.3 * (1 - 0.5 * 0.02 / 0.3) - 1e-3
    assert (st["rho"] >= 1000).all()
    # jitter is seeded and bounded
    g1 = api.dam_break_generate(cases.geometry("large", dx=0.02, jitter=0.01, seed=7))
    g2 = api.dam_break_generate(cases.geometry("large", dx=0.02, jitter=0.01, seed=7))
    g0 = api.dam_break_generate(cases.geometry("large", dx=0.02, jitter=0.0))
    assert np.array_equal(g1["pos"], g2["pos"])
    d = np.abs(g1["pos"] - g0["pos"])
    assert d.max() <= 0.01 * 0.02 * 1.01 and d.max() > 0


def test_obstacle_particles(sphlib):
    from tmp_sph_gb300 import api, cases
    st = api.dam_break_generate(cases.geometry("obstacle", dx=0.02))
    rig = st["pos"][st["type"] == api.SPH_TYPE_RIGID]
    assert len(rig) == 8 * 20 * 8
    assert rig[:, 0].min() > 2.32 and rig[:, 0].max() < 2.48 and rig[:, 2].max() < 0.16


def test_dat_roundtrip(sphlib, tmp_path):
    """The seven ini_fluid files (src/io/io.cu:10-111) written and read back."""
    from tmp_sph_gb300 import api, cases
    st = api.dam_break_generate(cases.geometry("small", dx=0.04))
    api.write_dat(str(tmp_path), st)
    for f in ("h_pos.dat", "h_vel.dat", "h_ac.dat", "rhop.dat", "p.dat", "particle_type.dat",
              "particle_zone.dat"):
        assert (tmp_path / f).exists()
    back = api.read_dat(str(tmp_path), len(st["rho"]))
    for k in ("pos", "vel", "rho", "p", "type"):
        assert np.array_equal(back[k], st[k]), k
    assert (back["zone"] == 0).all() and (back["ac"] == 0).all()


def test_library_fails_loudly_when_missing(tmp_path, monkeypatch):
    from tmp_sph_gb300 import api
    monkeypatch.setattr(api, "LIB_PATH", str(tmp_path / "missing.so"))
    monkeypatch.setattr(api, "_lib", None)
    with pytest.raises(ImportError):
        api.lib()
