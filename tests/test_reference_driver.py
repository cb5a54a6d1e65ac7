"""The drop-in boundary against the reference's own host code (CPU: compile and link only).

1. The reference's driver (src/sph/sph_run.cu: main and its step loop) and its IO
   (src/io/io.cu), compiled from a temporary copy of its tree, link against libsph_gb300.so
   alone: the copy has the reference's own hot-path definitions removed (lib/mesh.cu and
   equation/ns.cu are left out, the PC_predictionD/PC_correctionD kernels and their host
   wrappers are cut from sph_run.cu) and gains the one call the library needs,
   sph_shim_set_reference_params(temps) after the cudaMemcpyToSymbol of src/sph/sph_run.cu:105.
   Every hot-path function the driver calls resolves to the library's shim.
2. The seven text files sph_write_dat writes are read by the reference's own ini_fluid
   (src/io/io.cu:6-111) and give the generator's arrays back byte for byte.

The reference tree is found at SPH_REFERENCE_DIR (oracle/ref_build.py); these tests skip
where it is absent (the GPU hosts).  Nothing is written into the reference tree: the copy and
the build live in a pytest temporary directory.
"""
from __future__ import annotations

import os
import shutil
import subprocess

import numpy as np
import pytest

HOT_PATH = ("calcHash(float*, int*, int*, int)", "sortParticles(int*, int*, int)",
            "reorder(float*, float*, float*, float*, int*, int*, float*, float*, float*, float*, "
            "int*, int*, int*, int*, int*, int*, int, SimParams*)",
            "recover(", "SPH_NS_simpleversion(", "PC_prediction(", "PC_correction(")


def _reference_src():
    from oracle import ref_build
    if not ref_build.reference_present():
        pytest.skip("reference sources absent (set SPH_REFERENCE_DIR)")
    return os.path.join(ref_build.REFERENCE, "src")


def _nvcc():
    from tmp_sph_gb300 import build
    try:
        return build.nvcc()
    except RuntimeError:
        pytest.skip("nvcc absent")


def _copy_tree(tmp_path) -> str:
    dst = os.path.join(str(tmp_path), "src")
    shutil.copytree(_reference_src(), dst)
    return dst


def _strip_integrator(path: str) -> None:
    """Cut the reference's integrator kernels and wrappers (the library's shim exports
    PC_prediction / PC_correction) and hand the host SimParams to the library once."""
    with open(path) as f:
        s = f.read()
    cut = s.index("__global__ void PC_predictionD(")
    s = s[:cut]
    call = "cudaMemcpyToSymbol(par, temps, sizeof(SimParams));"
    assert s.count(call) == 1
    s = s.replace(call, call + " sph_shim_set_reference_params("
                  "reinterpret_cast<const sph_ref_simparams*>(temps));")
    with open(path, "w") as f:
        f.write('#include "sph_gb300.h"\n' + s)


def test_reference_driver_links_against_library(sphlib, tmp_path):
    from tmp_sph_gb300 import build
    src = _copy_tree(tmp_path)
    _strip_integrator(os.path.join(src, "sph", "sph_run.cu"))
    exe = os.path.join(str(tmp_path), "sph_linked")
    libdir = os.path.dirname(build.LIB)
    cmd = [_nvcc(), "-O2", "-std=c++17", "-rdc=true", *build.ARCH, "-I", os.path.join(src, "header"),
           "-I", build.INCLUDE, os.path.join(src, "sph", "sph_run.cu"),
           os.path.join(src, "io", "io.cu"), "-L" + libdir, "-lsph_gb300",
           "-Xlinker", "-rpath," + libdir, "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    nm = subprocess.run(["nm", "-C", exe], capture_output=True, text=True).stdout
    undefined = [ln.split(" U ", 1)[1] for ln in nm.splitlines() if " U " in ln]
    for sym in HOT_PATH:
        assert any(u.startswith(sym) for u in undefined), f"{sym} not taken from the library"
    assert "sph_shim_set_reference_params" in undefined
    # the library defines every one of them
    lib_nm = subprocess.run(["nm", "-DC", "--defined-only", build.LIB], capture_output=True,
                            text=True).stdout
    for sym in HOT_PATH:
        assert sym in lib_nm, sym
    # and the executable resolves them from it (the dynamic loader finds every symbol)
    r = subprocess.run(["ldd", "-r", exe], capture_output=True, text=True)
    assert "undefined symbol" not in (r.stdout + r.stderr), (r.stdout + r.stderr)[-2000:]


READER = r"""
#include <cstdio>
#include <cstdlib>
#include <vector>
void ini_fluid(float* h_pos, float* h_vel, float* h_ac, float* rhop, float* p,
               int* particle_type, int* particle_zone, int np);
int main(int argc, char** argv) {
    if (argc != 3) return 2;
    const int np = std::atoi(argv[1]);
    std::vector<float> pos(3 * (size_t)np), vel(3 * (size_t)np), ac(3 * (size_t)np), rho(np), p(np);
    std::vector<int> type(np), zone(np);
    ini_fluid(pos.data(), vel.data(), ac.data(), rho.data(), p.data(), type.data(), zone.data(), np);
    FILE* f = std::fopen(argv[2], "wb");
    if (!f) return 3;
    std::fwrite(pos.data(), 4, pos.size(), f);
    std::fwrite(vel.data(), 4, vel.size(), f);
    std::fwrite(ac.data(), 4, ac.size(), f);
    std::fwrite(rho.data(), 4, rho.size(), f);
    std::fwrite(p.data(), 4, p.size(), f);
    std::fwrite(type.data(), 4, type.size(), f);
    std::fwrite(zone.data(), 4, zone.size(), f);
    return std::fclose(f) == 0 ? 0 : 4;
}
"""


def test_reference_ini_fluid_reads_generated_files(sphlib, tmp_path):
    from tmp_sph_gb300 import api, build, cases
    src = _copy_tree(tmp_path)
    main = os.path.join(str(tmp_path), "read_main.cu")
    with open(main, "w") as f:
        f.write(READER)
    exe = os.path.join(str(tmp_path), "read_dat")
    cmd = [_nvcc(), "-O2", "-std=c++17", *build.ARCH, "-I", os.path.join(src, "header"),
           os.path.join(src, "io", "io.cu"), main, "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    # a jittered case with walls, water and hydrostatic pressure (every array non-trivial)
    st, _ = cases.build("small", physics="config", dx=0.02, jitter=0.01)
    n = len(st["rho"])
    work = os.path.join(str(tmp_path), "run")
    os.makedirs(work)
    api.write_dat(work, st)
    out = os.path.join(str(tmp_path), "arrays.bin")
    r = subprocess.run([exe, str(n), out], cwd=work, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    raw = np.fromfile(out, dtype=np.uint8)
    assert raw.size == 4 * n * (3 + 3 + 3 + 1 + 1 + 1 + 1)
    f32 = raw.view(np.float32)
    o = 0

    def take(k):
        nonlocal o
        a = f32[o:o + k]
        o += k
        return a

    pos, vel, ac, rho, p = take(3 * n), take(3 * n), take(3 * n), take(n), take(n)
    typ, zone = raw.view(np.int32)[o:o + n], raw.view(np.int32)[o + n:o + 2 * n]
    # byte for byte: the text round trip loses nothing
    assert np.array_equal(pos.view(np.uint32), st["pos"].reshape(-1).view(np.uint32))
    assert np.array_equal(vel.view(np.uint32), st["vel"].reshape(-1).view(np.uint32))
    assert np.array_equal(rho.view(np.uint32), st["rho"].view(np.uint32))
    assert np.array_equal(p.view(np.uint32), st["p"].view(np.uint32))
    assert np.array_equal(typ, st["type"])
    assert not ac.any() and not zone.any()
