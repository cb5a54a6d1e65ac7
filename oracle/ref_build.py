"""Recipe for oracle/_ref: the reference solver's own kernels, compiled from its sources.
TEST INFRASTRUCTURE ONLY.

  build_fatbin()  — where the reference sources are present (this container): compiles the
                    reference's src/ tree (lib/mesh.cu, equation/ns.cu, sph/sph_run.cu with
                    its main renamed) as one translation unit into an sm_103a fatbin,
                    oracle/_ref/ref_src.fatbin.  Device code does not depend on the host CPU,
                    so the same file serves the aarch64 GPU hosts, where the sources are absent.
  build_harness() — anywhere with nvcc: compiles oracle/ref_harness.cu (this project's
                    driver-API loader) into oracle/_ref/libref_harness.so.

Nothing from the reference is copied: the unity file holds three #include lines that point
into the reference tree, and outputs go only to oracle/_ref/ (git-ignored).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
# Where the reference's source tree is: SPH_REFERENCE_DIR, else the checkout this recipe was
# written against.  Nothing that runs on a GPU host reads it (the fatbins built here travel).
REFERENCE = os.environ.get("SPH_REFERENCE_DIR", "/root/reference")
FATBIN = os.path.join(OUT, "ref_src.fatbin")
HARNESS = os.path.join(OUT, "libref_harness.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

# The reference's six code trees: the baseline and its five optimisation snapshots.  Flags
# follow each tree's CMakeLists.txt (v0-v4 cap registers at 64; v3 and v4 use std::vector
# without including it; v4 adds lib/mem.cu).
VERSIONS = {
    "src": ("src", []),
    "v0": ("opt_src_v0", ["-maxrregcount", "64"]),
    "v1": ("opt_src_v1", ["-maxrregcount", "64"]),
    "v2": ("opt_src_v2", ["-maxrregcount", "64"]),
    "v3": ("opt_src_v3", ["-maxrregcount", "64"]),
    "v4": ("opt_src_v4", ["-maxrregcount", "64"]),
}


def fatbin_path(version: str) -> str:
    return FATBIN if version == "src" else os.path.join(OUT, f"ref_{version}.fatbin")


def nvcc() -> str:
    for c in ("/usr/local/cuda/bin/nvcc", shutil.which("nvcc") or ""):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def reference_present() -> bool:
    return os.path.isdir(os.path.join(REFERENCE, "src", "equation"))


def require_reference() -> str:
    """The reference tree, or a clear error naming the variable that locates it."""
    if not reference_present():
        raise FileNotFoundError(
            f"reference sources not found at {REFERENCE} (expected src/equation there); "
            "set SPH_REFERENCE_DIR to the ZZPHUB/tmp_sph checkout")
    return REFERENCE


def build_fatbin(force: bool = False, version: str = "src") -> str | None:
    out = fatbin_path(version)
    if not reference_present():
        return out if os.path.exists(out) else None
    if os.path.exists(out) and not force:
        return out
    tree, flags = VERSIONS[version]
    os.makedirs(OUT, exist_ok=True)
    src = os.path.join(REFERENCE, tree)
    unity = os.path.join(OUT, f"unity_{version}.cu")
    with open(unity, "w") as f:
        f.write('#define main reference_main\n#include "lib/mesh.cu"\n'
                '#include "equation/ns.cu"\n#include "sph/sph_run.cu"\n')
        if os.path.exists(os.path.join(src, "lib", "mem.cu")):
            f.write('#include "lib/mem.cu"\n')
    cmd = [nvcc(), "-fatbin", *ARCH, "-O3", "-w", "-include", "vector", *flags, "-I" + src,
           "-I" + os.path.join(src, "header"), unity, "-o", out + ".tmp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"reference fatbin build failed ({version}):\n{r.stderr[-3000:]}")
    os.replace(out + ".tmp", out)
    return out


def build_all_fatbins(force: bool = False) -> dict:
    return {v: build_fatbin(force, v) for v in VERSIONS}


def build_harness(force: bool = False) -> str:
    src = os.path.join(HERE, "ref_harness.cu")
    if (os.path.exists(HARNESS) and not force
            and os.path.getmtime(HARNESS) > os.path.getmtime(src)
            and _machine_stamp_ok()):
        return HARNESS
    os.makedirs(OUT, exist_ok=True)
    cmd = [nvcc(), *ARCH, "-O2", "-std=c++17", "-shared", "-Xcompiler", "-fPIC", src,
           "-o", HARNESS + ".tmp", "-lcuda"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"harness build failed:\n{r.stderr[-3000:]}")
    os.replace(HARNESS + ".tmp", HARNESS)
    with open(os.path.join(OUT, "harness.machine"), "w") as f:
        f.write(os.uname().machine)
    return HARNESS


def _machine_stamp_ok() -> bool:
    p = os.path.join(OUT, "harness.machine")
    return os.path.exists(p) and open(p).read().strip() == os.uname().machine


def build(force: bool = False) -> dict:
    return {"fatbins": build_all_fatbins(force), "harness": build_harness(force)}


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
