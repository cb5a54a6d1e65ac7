"""ctypes binding of the CPU oracle (libsph_oracle.so).  TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline and reference legs use this
module, as the checker; the product never imports it.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build_oracle

F3 = C.c_float * 3
I3 = C.c_int * 3


class OrParams(C.Structure):
    _fields_ = [
        ("num_particles", C.c_int), ("num_boundary", C.c_int), ("dt", C.c_float),
        ("gravity", C.c_float), ("cell_size", C.c_float), ("grid_min", F3), ("grid_max", F3),
        ("grid_dim", I3), ("num_cells", C.c_int), ("dx", C.c_float), ("h", C.c_float),
        ("kh", C.c_float), ("eta", C.c_float), ("delta", C.c_float), ("alpha", C.c_float),
        ("adh", C.c_float), ("mass", C.c_float), ("rho0", C.c_float), ("cs", C.c_float),
        ("eos", C.c_int), ("tait_gamma", C.c_float), ("tait_b", C.c_float),
        ("clamp_density", C.c_int), ("escape_min", F3), ("escape_max", F3),
        ("escape_park", F3), ("park_inactive", C.c_int),
        ("reserved", C.c_int * 7),
    ]

    def as_dict(self) -> dict:
        out = {}
        for name, _ in self._fields_:
            v = getattr(self, name)
            out[name] = list(v) if hasattr(v, "__len__") else v
        return out


class OrDamBreak(C.Structure):
    """or_dam_break (sph_oracle.h): the seeded dam-break generator's description."""
    _fields_ = [
        ("dx", C.c_float), ("tank", F3), ("block", F3), ("wall_layers", C.c_int),
        ("has_obstacle", C.c_int), ("obstacle_min", F3), ("obstacle_max", F3),
        ("jitter", C.c_float), ("seed", C.c_ulonglong), ("hydrostatic", C.c_int),
        ("rho0", C.c_float), ("gravity", C.c_float), ("cs", C.c_float), ("eos", C.c_int),
        ("tait_gamma", C.c_float),
    ]


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        path = build_oracle.build()
        L = C.CDLL(path)
        P = C.c_void_p
        I = C.c_int
        PP = C.POINTER(OrParams)
        protos = {
            "or_params_reference": (None, [C.c_float] * 4 + [I, I, PP]),
            "or_params_general": (None, [C.c_float, C.c_double, C.c_float, C.c_float, C.c_float,
                                         C.c_float, C.c_float, C.c_float, C.c_float, I, C.c_float,
                                         P, P, C.c_double, C.c_double, I, I, PP]),
            "or_sort_particles": (None, [P, P, I]),
            "or_set_threads": (I, [I]),
            "or_dam_break_count": (C.c_long, [C.POINTER(OrDamBreak), C.POINTER(C.c_long)]),
            "or_dam_break_generate": (I, [C.POINTER(OrDamBreak), P, P, P, P, P, C.c_long]),
        }
        for suf in ("_f32", "_f64"):
            protos.update({
                "or_calc_hash" + suf: (None, [PP, P, P, P, I]),
                "or_reorder" + suf: (None, [PP] + [P] * 16 + [I]),
                "or_recover" + suf: (None, [P, P, P, P, I] + [P] * 9),
                "or_sph_ns" + suf: (None, [PP] + [P] * 9 + [I, P, P, P, P]),
                "or_pc_prediction" + suf: (None, [PP] + [P] * 10 + [I, P]),
                "or_pc_correction" + suf: (None, [PP] + [P] * 10 + [I, P]),
                "or_run" + suf: (I, [PP, P, P, P, P, P, I, I]),
            })
        for name, (res, args) in protos.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _p(a):
    if a is None:
        return None
    assert isinstance(a, np.ndarray) and a.flags["C_CONTIGUOUS"], "oracle takes contiguous numpy"
    return a.ctypes.data


def set_threads(n: int) -> int:
    return lib().or_set_threads(n)


def params_reference(dx, vlx, vly, vlz, np_=0, nb=0) -> OrParams:
    p = OrParams()
    lib().or_params_reference(dx, vlx, vly, vlz, np_, nb, C.byref(p))
    return p


def params_general(dx, h_factor, rho0, cs, gravity, delta, alpha, dt, cfl, eos, tait_gamma,
                   dmin, dmax, pad, cell_factor, np_, nb) -> OrParams:
    p = OrParams()
    a = np.asarray(dmin, np.float32)
    b = np.asarray(dmax, np.float32)
    lib().or_params_general(dx, h_factor, rho0, cs, gravity, delta, alpha, dt, cfl, eos,
                            tait_gamma, _p(a), _p(b), pad, cell_factor, np_, nb, C.byref(p))
    return p


def params_like(src) -> OrParams:
    """Copy a layout-compatible parameter struct (same field names) into OrParams."""
    p = OrParams()
    for name, _ in OrParams._fields_:
        setattr(p, name, getattr(src, name))
    return p


def dam_break_generate(d: OrDamBreak) -> dict:
    """Host arrays of a generated dam break (walls, obstacle, water): pos/vel (n,3) f32,
    rho/p (n,) f32, type (n,) i32, plus n_fluid and n_boundary."""
    nf = C.c_long(0)
    n = lib().or_dam_break_count(C.byref(d), C.byref(nf))
    st = {"pos": np.zeros((n, 3), np.float32), "vel": np.zeros((n, 3), np.float32),
          "rho": np.zeros(n, np.float32), "p": np.zeros(n, np.float32),
          "type": np.zeros(n, np.int32)}
    rc = lib().or_dam_break_generate(C.byref(d), _p(st["pos"]), _p(st["vel"]), _p(st["rho"]),
                                     _p(st["p"]), _p(st["type"]), n)
    if rc != 0:
        raise RuntimeError("oracle generator: particle count mismatch")
    st["n_fluid"] = int(nf.value)
    st["n_boundary"] = int(n - nf.value)
    return st


def sort_particles(hash_: np.ndarray, index: np.ndarray) -> None:
    lib().or_sort_particles(_p(hash_), _p(index), len(hash_))


def _suffix(a: np.ndarray) -> str:
    return "_f64" if a.dtype == np.float64 else "_f32"


def calc_hash(P: OrParams, pos: np.ndarray):
    n = pos.shape[0]
    h = np.zeros(n, np.int32)
    idx = np.zeros(n, np.int32)
    getattr(lib(), "or_calc_hash" + _suffix(pos))(C.byref(P), _p(pos), _p(h), _p(idx), n)
    return h, idx


def cell_list(P: OrParams, st: dict):
    """Hash, stable sort and reorder of a state in original order (src/lib/mesh.cu:26-159).
    Returns the sorted state plus hash, index, cell_start, cell_end."""
    pos = st["pos"]
    n = pos.shape[0]
    dt = pos.dtype
    h, idx = calc_hash(P, pos)
    sort_particles(h, idx)
    out = {"pos": np.zeros_like(pos), "vel": np.zeros_like(st["vel"]),
           "rho": np.zeros(n, dt), "p": np.zeros(n, dt), "type": np.zeros(n, np.int32),
           "hash": h, "index": idx,
           "cell_start": np.zeros(P.num_cells, np.int32),
           "cell_end": np.full(P.num_cells, -7, np.int32)}
    getattr(lib(), "or_reorder" + _suffix(pos))(
        C.byref(P), _p(pos), _p(st["vel"]), _p(st["rho"]), _p(st["p"]), _p(st["type"]), None,
        _p(out["pos"]), _p(out["vel"]), _p(out["rho"]), _p(out["p"]), _p(out["type"]), None,
        _p(h), _p(idx), _p(out["cell_start"]), _p(out["cell_end"]), n)
    return out


def sph_ns(P: OrParams, s: dict) -> dict:
    """Both neighbour kernels on a sorted state (modifies s['p'], s['rho'] of walls)."""
    n = s["pos"].shape[0]
    dt = s["pos"].dtype
    r = {"rho_dt": np.zeros(n, dt), "vel_dt": np.zeros((n, 3), dt), "dofv": np.zeros(n, dt),
         "rhop_sum": np.zeros(n, dt), "w_sum": np.zeros(n, dt)}
    getattr(lib(), "or_sph_ns" + _suffix(s["pos"]))(
        C.byref(P), _p(s["pos"]), _p(s["vel"]), _p(s["rho"]), _p(s["p"]), _p(s["type"]),
        _p(r["rho_dt"]), _p(r["vel_dt"]), _p(s["cell_start"]), _p(s["cell_end"]), n, _p(s["hash"]),
        _p(r["dofv"]), _p(r["rhop_sum"]), _p(r["w_sum"]))
    return r


def pc_prediction(P, s, rates, tmp) -> None:
    n = s["pos"].shape[0]
    getattr(lib(), "or_pc_prediction" + _suffix(s["pos"]))(
        C.byref(P), _p(s["pos"]), _p(s["vel"]), _p(s["rho"]), _p(s["p"]), _p(rates["rho_dt"]),
        _p(rates["vel_dt"]), _p(s["index"]), _p(tmp["pos"]), _p(tmp["vel"]), _p(tmp["rho"]), n,
        _p(s["type"]))


def pc_correction(P, s, rates, tmp) -> None:
    n = s["pos"].shape[0]
    getattr(lib(), "or_pc_correction" + _suffix(s["pos"]))(
        C.byref(P), _p(s["pos"]), _p(s["vel"]), _p(s["rho"]), _p(s["p"]), _p(rates["rho_dt"]),
        _p(rates["vel_dt"]), _p(s["index"]), _p(tmp["pos"]), _p(tmp["vel"]), _p(tmp["rho"]), n,
        _p(s["type"]))


def run(P: OrParams, st: dict, nsteps: int, dtype=np.float32) -> dict:
    """nsteps of the reference step loop on a copy of st (original order)."""
    out = {k: np.array(st[k], dtype=dtype, copy=True) for k in ("pos", "vel", "rho", "p")}
    out["type"] = np.array(st["type"], np.int32, copy=True)
    n = out["pos"].shape[0]
    fn = getattr(lib(), "or_run" + ("_f64" if dtype == np.float64 else "_f32"))
    rc = fn(C.byref(P), _p(out["pos"]), _p(out["vel"]), _p(out["rho"]), _p(out["p"]),
            _p(out["type"]), n, nsteps)
    if rc != 0:
        raise MemoryError("oracle allocation failed")
    return out
