"""Named dam-break cases: geometry (for the seeded generator) and physics (for the parameter
derivation).

Geometries are the five benchmark workloads of this project:

  small      tank 1.0 x 0.5 x 0.6 m, water 0.4 x 0.5 x 0.3 m at x = 0, dx 0.01  (133,968 particles)
  large      same tank and water, dx 0.0025, +-0.01 dx jitter                  (4,963,548)
  precision  same tank and water, dx 0.005                                     (765,828)
  obstacle   tank 3.22 x 1.0 x 1.0, water 1.2 x 1.0 x 0.55, rigid box
             0.16 x 0.4 x 0.16 centred at x = 2.4, y = 0.5 on the floor, dx 0.005
  refcase    the reference's own hard-coded tank 3.221 x 1 x 1, water 1.228 x 1 x 0.55
             (src/sph/sph_run.cu:11-13) at a chosen dx

and batch(): 64 independent dam breaks in the 1.0 x 0.5 x 0.6 m tank at dx 0.005, water blocks
of width U[0.2, 0.6] m and height U[0.15, 0.45] m (about 120k-1.08M fluid particles each,
49M particles in all) for the batched solver.

Physics variants:

  "config"     h = 1.3 dx, rho0 1000, c0 = 10 sqrt(2 g 0.3), Tait gamma 7, delta 0.1,
               alpha 0.02, g = -9.81, dt = 0.25 h / c0
  "reference"  the reference's hard-coded constants (src/sph/sph_run.cu:12-16,60-101):
               h = 1.5 dx, cs 25, linear EOS, delta 0.2, alpha 0.05, dt 2e-4
"""
from __future__ import annotations

import math

from . import api

C0 = 10.0 * math.sqrt(2.0 * 9.81 * 0.3)  # 24.26 m/s

_GEOM = {
    "small": dict(dx=0.01, tank=(1.0, 0.5, 0.6), block=(0.4, 0.5, 0.3), jitter=0.0),
    "large": dict(dx=0.0025, tank=(1.0, 0.5, 0.6), block=(0.4, 0.5, 0.3), jitter=0.01),
    "precision": dict(dx=0.005, tank=(1.0, 0.5, 0.6), block=(0.4, 0.5, 0.3), jitter=0.0),
    "obstacle": dict(dx=0.005, tank=(3.22, 1.0, 1.0), block=(1.2, 1.0, 0.55), jitter=0.0,
                     obstacle=((2.32, 0.3, 0.0), (2.48, 0.7, 0.16))),
    "refcase": dict(dx=0.01, tank=(3.221, 1.0, 1.0), block=(1.228, 1.0, 0.55), jitter=0.0),
}

CASES = tuple(_GEOM)


def geometry(name: str, *, dx: float | None = None, block=None, tank=None,
             jitter: float | None = None, seed: int = 20240611, physics: str = "config",
             hydrostatic: bool = True) -> api.SphDamBreak:
    g = dict(_GEOM[name])
    if dx is not None:
        g["dx"] = dx
    if block is not None:
        g["block"] = tuple(block)
    if tank is not None:
        g["tank"] = tuple(tank)
    if jitter is not None:
        g["jitter"] = jitter
    d = api.SphDamBreak()
    d.dx = g["dx"]
    d.tank = api.F3(*g["tank"])
    d.block = api.F3(*g["block"])
    d.wall_layers = 3
    obs = g.get("obstacle")
    d.has_obstacle = 1 if obs else 0
    if obs:
        d.obstacle_min = api.F3(*obs[0])
        d.obstacle_max = api.F3(*obs[1])
    d.jitter = g["jitter"]
    d.seed = seed
    d.hydrostatic = 1 if hydrostatic else 0
    d.rho0 = 1000.0
    d.gravity = -9.81
    if physics == "config":
        d.cs, d.eos, d.tait_gamma = C0, api.SPH_EOS_TAIT, 7.0
    else:
        d.cs, d.eos, d.tait_gamma = 25.0, api.SPH_EOS_LINEAR, 7.0
    return d


def lattice_extent(length: float, dx: float) -> float:
    """Extent actually covered by the generator's lattice along one tank axis
    (round(length/dx) cells of width dx)."""
    return math.floor(float(length) / float(dx) + 0.5) * float(dx)


def config(d: api.SphDamBreak, physics: str = "config", n: int = 0, nb: int = 0,
           cell_factor: float = 1.0) -> api.SphConfig:
    """Physics configuration for a generated geometry: grid = tank padded by 0.1 m (more when
    the wall layers are thicker than that), escape box = the lattice tank, 5 cm above its rim,
    parking point 8 cm below the floor as in the reference."""
    c = api.SphConfig()
    c.dx = d.dx
    c.rho0 = 1000.0
    c.gravity = -9.81
    if physics == "config":
        c.h_factor, c.cs, c.delta, c.alpha = 1.3, C0, 0.1, 0.02
        c.dt, c.cfl, c.eos = 0.0, 0.25, api.SPH_EOS_TAIT
    elif physics == "reference":
        c.h_factor, c.cs, c.delta, c.alpha = 1.5, 25.0, 0.2, 0.05
        c.dt, c.cfl, c.eos = 2e-4, 0.0, api.SPH_EOS_LINEAR
    else:
        raise ValueError(physics)
    c.tait_gamma = 7.0
    tank = [lattice_extent(t, d.dx) for t in d.tank]
    c.domain_min = api.F3(0.0, 0.0, 0.0)
    c.domain_max = api.F3(*tank)
    # the wall layers (and a cell of margin) must stay inside the padded grid
    c.pad = max(0.1, (d.wall_layers + 1.5) * float(d.dx))
    c.cell_factor = cell_factor
    c.escape_min = api.F3(0.0, 0.0, 0.0)
    c.escape_max = api.F3(tank[0], tank[1], tank[2] + 0.05)
    c.escape_park = api.F3(0.0, 0.5 * tank[1], -0.08 - (c.pad - 0.1))
    c.num_particles = n
    c.num_boundary = nb
    c.clamp_density = 1
    return c


def batch(n_inst: int = 64, *, seed: int = 20240611, dx: float = 0.005,
          tank=(1.0, 0.5, 0.6), width=(0.2, 0.6), height=(0.15, 0.45),
          jitter: float = 0.0) -> tuple[list, api.SphParams]:
    """Independent dam breaks for one batched solver: the same tank, water blocks of width
    U[width] and height U[height] drawn from `seed` (full tank breadth, at x = 0).  They share
    one parameter set, so the speed of sound is set by the tallest column,
    c0 = 10 sqrt(2 g H_max), and dt = 0.25 h / c0 for all.  Returns (states, params)."""
    import numpy as np
    rng = np.random.default_rng(seed)
    widths = rng.uniform(width[0], width[1], n_inst)
    heights = rng.uniform(height[0], height[1], n_inst)
    cs = 10.0 * math.sqrt(2.0 * 9.81 * float(heights.max()))
    states, nb = [], 0
    d = None
    for b in range(n_inst):
        d = geometry("precision", dx=dx, tank=tank, block=(float(widths[b]), tank[1],
                                                         float(heights[b])),
                     jitter=jitter, seed=seed + b)
        d.cs = cs
        st = api.dam_break_generate(d)
        st["geometry"] = d
        st["block"] = (float(widths[b]), float(heights[b]))
        states.append(st)
        nb += st["n_boundary"]
    n = sum(len(st["rho"]) for st in states)
    c = config(d, "config", n, nb)
    c.cs = cs
    return states, api.params_derive(c)


def build(name: str, physics: str = "config", **kw) -> tuple[dict, api.SphParams]:
    """Generate a case: (host state dict, derived parameters)."""
    d = geometry(name, physics=physics, **kw)
    st = api.dam_break_generate(d)
    n = st["n_fluid"] + st["n_boundary"]
    # config() keeps the reference's 0.1 m pad unless the wall layers are thicker than that
    # (coarse test spacings), so every particle hashes into the grid
    p = api.params_derive(config(d, physics, n, st["n_boundary"]))
    st["geometry"] = d
    return st, p
