"""Build the CPU oracle (libsph_oracle.so) with gcc.  TEST INFRASTRUCTURE.

gcc -O2 -std=c11 -fopenmp -ffp-contract=off: every float and double operation rounded on
its own (no fused multiply-add), OpenMP over particles for the timed CPU baseline.
"""
from __future__ import annotations

import hashlib
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "libsph_oracle.so")
SOURCES = ["sph_oracle.c", "sph_oracle_gen.c"]
DEPS = ["sph_oracle.h", "sph_oracle_phys.inc"]
FLAGS = ["-O2", "-std=c11", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", "-Wall"]


def build(force: bool = False) -> str:
    h = hashlib.sha256()
    for f in SOURCES + DEPS:
        with open(os.path.join(HERE, f), "rb") as fh:
            h.update(fh.read())
    h.update(" ".join(FLAGS).encode() + os.uname().machine.encode())
    stamp = os.path.join(HERE, ".oracle_stamp")
    dig = h.hexdigest()
    if not force and os.path.exists(LIB) and os.path.exists(stamp):
        with open(stamp) as fh:
            if fh.read().strip() == dig:
                return LIB
    tmp = LIB + ".tmp"
    cmd = ["gcc", *FLAGS, *[os.path.join(HERE, s) for s in SOURCES], "-o", tmp, "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    with open(stamp, "w") as fh:
        fh.write(dig)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
