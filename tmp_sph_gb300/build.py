"""Build the CUDA library libsph_gb300.so in-tree for sm_103a (nvcc, no cmake).

Every translation unit is compiled in parallel with one -gencode (compute_103a -> sm_103a),
-O3 -lineinfo, then linked into a shared library next to this file.  Usage:

    python -m tmp_sph_gb300.build            # build if sources changed
    python -m tmp_sph_gb300.build --force    # rebuild
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
OBJDIR = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libsph_gb300.so")

SOURCES = [
    "lib/mesh.cu",
    "lib/sort_noalloc.cu",
    "equation/ns.cu",
    "equation/ns_groups.cu",
    "sph/integrator.cu",
    "sph/solver.cu",
    "sph/params.cpp",
    "sph/ref_shim.cu",
    "io/dam_break.cpp",
    "io/probes.cu",
    "io/vtk.cpp",
    "io/peak.cu",
]
HEADERS = ["header/sph_device.cuh", "header/sph_internal.h", "equation/ns_pair.cuh"]

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CFLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
          "--expt-relaxed-constexpr", "-I" + INCLUDE, "-I" + os.path.join(CSRC, "header")]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def cuda_libdir() -> str:
    base = os.path.dirname(os.path.dirname(os.path.realpath(nvcc())))
    for sub in ("lib64", "lib", "targets/sbsa-linux/lib", "targets/x86_64-linux/lib"):
        d = os.path.join(base, sub)
        if os.path.exists(os.path.join(d, "libcudart.so")):
            return d
    return os.path.join(base, "lib64")


def _digest(extra: list[str]) -> str:
    h = hashlib.sha256()
    for rel in SOURCES + HEADERS:
        with open(os.path.join(CSRC, rel), "rb") as f:
            h.update(f.read())
    with open(os.path.join(INCLUDE, "sph_gb300.h"), "rb") as f:
        h.update(f.read())
    h.update(" ".join(ARCH + CFLAGS + extra).encode())
    h.update(os.uname().machine.encode())
    return h.hexdigest()


def _compile(src: str, extra: list[str]) -> str:
    obj = os.path.join(OBJDIR, src.replace("/", "_") + ".o")
    cmd = [nvcc(), *ARCH, *CFLAGS, *extra, "-x", "cu", "-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj


def build(force: bool = False, verbose: bool = False, extra: list[str] | None = None) -> str:
    """Compile the library if any source changed; return the path of the .so."""
    extra = list(extra or [])
    os.makedirs(OBJDIR, exist_ok=True)
    stamp = os.path.join(OBJDIR, "stamp")
    dig = _digest(extra)
    if not force and os.path.exists(LIB) and os.path.exists(stamp):
        with open(stamp) as f:
            if f.read().strip() == dig:
                return LIB
    with cf.ThreadPoolExecutor(max_workers=min(len(SOURCES), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra), SOURCES))
    libdir = cuda_libdir()
    tmp = LIB + ".tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-cudart", "shared", "-o", tmp, *objs,
           "-Xlinker", "-rpath," + libdir, "-L" + libdir]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    with open(stamp, "w") as f:
        f.write(dig)
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True,
          extra=["-Xptxas", "-v"] if "--ptxas-v" in sys.argv else None)
