"""The benchmark workloads built on the oracle side alone.  TEST INFRASTRUCTURE.

bench.py's reference leg (the oracle's restatement of the reference step loop on the host
cores) and the tests build their inputs here, with the oracle's own generator
(sph_oracle_gen.c) and parameter derivation (or_params_general, the derivation of
src/sph/sph_run.cu:60-101 with the constants as inputs), so no product library is loaded.
The case table and the physics constants are the same as the product's workload definitions
(tmp_sph_gb300/cases.py); tests/test_oracle.py checks that both give the same state and the
same parameters, bit for bit.

  small      tank 1.0 x 0.5 x 0.6 m, water 0.4 x 0.5 x 0.3 m at x = 0, dx 0.01  (133,968 particles)
  large      same tank and water, dx 0.0025, +-0.01 dx jitter                  (4,963,548)
  precision  same tank and water, dx 0.005                                     (765,828)
  obstacle   tank 3.22 x 1.0 x 1.0, water 1.2 x 1.0 x 0.55, rigid box
             0.16 x 0.4 x 0.16 centred at x = 2.4, y = 0.5 on the floor, dx 0.005
  refcase    the reference's tank 3.221 x 1 x 1 and water 1.228 x 1 x 0.55
             (src/sph/sph_run.cu:11-13)
"""
from __future__ import annotations

import math

from . import oracle as O

C0 = 10.0 * math.sqrt(2.0 * 9.81 * 0.3)  # 24.26 m/s

GEOM = {
    "small": dict(dx=0.01, tank=(1.0, 0.5, 0.6), block=(0.4, 0.5, 0.3), jitter=0.0),
    "large": dict(dx=0.0025, tank=(1.0, 0.5, 0.6), block=(0.4, 0.5, 0.3), jitter=0.01),
    "precision": dict(dx=0.005, tank=(1.0, 0.5, 0.6), block=(0.4, 0.5, 0.3), jitter=0.0),
    "obstacle": dict(dx=0.005, tank=(3.22, 1.0, 1.0), block=(1.2, 1.0, 0.55), jitter=0.0,
                     obstacle=((2.32, 0.3, 0.0), (2.48, 0.7, 0.16))),
    "refcase": dict(dx=0.01, tank=(3.221, 1.0, 1.0), block=(1.228, 1.0, 0.55), jitter=0.0),
}

SEED = 20240611


def geometry(name: str, physics: str = "config", dx: float | None = None,
             seed: int = SEED) -> O.OrDamBreak:
    g = dict(GEOM[name])
    if dx is not None:
        g["dx"] = dx
    d = O.OrDamBreak()
    d.dx = g["dx"]
    d.tank = O.F3(*g["tank"])
    d.block = O.F3(*g["block"])
    d.wall_layers = 3
    obs = g.get("obstacle")
    d.has_obstacle = 1 if obs else 0
    if obs:
        d.obstacle_min = O.F3(*obs[0])
        d.obstacle_max = O.F3(*obs[1])
    d.jitter = g["jitter"]
    d.seed = seed
    d.hydrostatic = 1
    d.rho0 = 1000.0
    d.gravity = -9.81
    if physics == "config":
        d.cs, d.eos, d.tait_gamma = C0, 1, 7.0
    else:
        d.cs, d.eos, d.tait_gamma = 25.0, 0, 7.0
    return d


def lattice_extent(length: float, dx: float) -> float:
    return math.floor(float(length) / float(dx) + 0.5) * float(dx)


def params(d: O.OrDamBreak, physics: str, n: int, nb: int) -> O.OrParams:
    """Grid = lattice tank padded by 0.1 m (more when the wall layers are thicker), escape box
    = the lattice tank 5 cm above its rim, parking point 8 cm below the floor."""
    tank = [lattice_extent(t, d.dx) for t in d.tank]
    pad = max(0.1, (d.wall_layers + 1.5) * float(d.dx))
    if physics == "config":
        hf, cs, delta, alpha, dt, cfl, eos = 1.3, C0, 0.1, 0.02, 0.0, 0.25, 1
    elif physics == "reference":
        hf, cs, delta, alpha, dt, cfl, eos = 1.5, 25.0, 0.2, 0.05, 2e-4, 0.0, 0
    else:
        raise ValueError(physics)
    P = O.params_general(d.dx, hf, 1000.0, cs, -9.81, delta, alpha, dt, cfl, eos, 7.0,
                         [0.0, 0.0, 0.0], tank, pad, 1.0, n, nb)
    P.escape_min = O.F3(0.0, 0.0, 0.0)
    P.escape_max = O.F3(tank[0], tank[1], tank[2] + 0.05)
    P.escape_park = O.F3(0.0, 0.5 * tank[1], -0.08 - (pad - 0.1))
    P.clamp_density = 1
    return P


def build(name: str, physics: str = "config", **kw) -> tuple[dict, O.OrParams]:
    """(host state dict, oracle parameters) of a named workload."""
    d = geometry(name, physics, **kw)
    st = O.dam_break_generate(d)
    n = st["n_fluid"] + st["n_boundary"]
    return st, params(d, physics, n, st["n_boundary"])
