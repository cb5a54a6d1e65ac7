"""Python handle on the reference's own compiled kernels (oracle/_ref).  TEST INFRASTRUCTURE.

RefHarness runs the reference solver's src/ kernels on the GPU with the reference's launch
shapes, on torch CUDA buffers, to generate golden fixtures and to time the reference's CUDA
step loop.  Needs oracle/_ref/ref_src.fatbin (built where the reference sources are, see
ref_build.py) and builds the harness library itself.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import ref_build

F = C.c_float
I = C.c_int


class RefSimParams(C.Structure):
    """Byte layout of the reference's SimParams (src/header/data_struct.cuh:4-44)."""
    _fields_ = (
        [("timeStep", F), ("time", F), ("numParticles", I), ("boundary_p_num", I), ("gravity", F)]
        + [(n, F) for n in ("gridSize", "gridxmin", "gridymin", "gridzmin", "gridxmax", "gridymax",
                            "gridzmax")]
        + [(n, I) for n in ("gridxdim", "gridydim", "gridzdim", "numCells", "hash_max", "hash_min")]
        + [(n, F) for n in ("pre_set_domain_x_min", "pre_set_domain_x_max", "pre_set_domain_y_min",
                            "pre_set_domain_y_max", "pre_set_domain_z_min", "pre_set_domain_z_max",
                            "particleR", "h", "kh", "eta", "delta", "afa", "SpikyKern", "LapKern",
                            "Poly6Kern", "minDist", "particleMass", "restDensity", "viscosity",
                            "stiffness", "cs", "adh", "namuta_threshold_1", "namuta_threshold_2",
                            "CFL", "Ma", "conc_0", "conc_t", "PST_R", "PST_n", "w_deltar")]
        + [(n, I) for n in ("ngp", "nnode", "n_edge", "num_vp", "max_nspnode", "nele")]
        + [("mat_para", F * 3)]
    )


def simparams_from(P, n: int) -> RefSimParams:
    """The reference's SimParams for oracle parameters P (the fields its kernels read), with
    hash_max as src/sph/sph_run.cu:92 sets it."""
    r = RefSimParams()
    gx, gy, gz = P.grid_dim[0], P.grid_dim[1], P.grid_dim[2]
    r.timeStep, r.numParticles, r.boundary_p_num, r.gravity = P.dt, n, P.num_boundary, P.gravity
    r.gridSize = P.cell_size
    r.gridxmin, r.gridymin, r.gridzmin = P.grid_min[0], P.grid_min[1], P.grid_min[2]
    r.gridxmax, r.gridymax, r.gridzmax = P.grid_max[0], P.grid_max[1], P.grid_max[2]
    r.gridxdim, r.gridydim, r.gridzdim, r.numCells = gx, gy, gz, P.num_cells
    r.hash_max, r.hash_min = gx * gy * gz + gx * gy + gx, 0
    r.particleR, r.h, r.kh, r.eta, r.delta, r.afa = P.dx, P.h, P.kh, P.eta, P.delta, P.alpha
    r.particleMass, r.restDensity, r.cs, r.adh = P.mass, P.rho0, P.cs, P.adh
    return r


class RefHarness:
    def __init__(self):
        fat = ref_build.FATBIN
        if not os.path.exists(fat):
            raise FileNotFoundError(f"{fat} missing (built from the reference sources)")
        self.L = C.CDLL(ref_build.build_harness())
        self.L.refh_error.restype = C.c_char_p
        self.L.refh_params_bytes.restype = C.c_size_t
        self._ok(self.L.refh_load(fat.encode()))
        self.n = 0

    def _ok(self, rc):
        if rc != 0:
            raise RuntimeError("reference harness: " + self.L.refh_error().decode())

    def set_params(self, P, n: int) -> None:
        r = simparams_from(P, n)
        assert self.L.refh_params_bytes() == C.sizeof(r)
        self._ok(self.L.refh_set_params(C.byref(r), C.c_size_t(C.sizeof(r)), P.num_cells))
        self.P, self.n = P, n

    # device buffers ------------------------------------------------------------
    @staticmethod
    def _p(t):
        return C.c_void_p(t.data_ptr()) if t is not None else C.c_void_p(0)

    def calc_hash(self, pos, h, idx):
        self._ok(self.L.refh_calc_hash(self._p(pos), self._p(h), self._p(idx), self.n))

    def sort(self, h, idx):
        self._ok(self.L.refh_sort(self._p(h), self._p(idx), self.n))

    def reorder(self, d, s, h, idx, cs, ce):
        p = self._p
        self._ok(self.L.refh_reorder(p(d["pos"]), p(d["vel"]), p(d["rho"]), p(d["p"]), p(d["type"]),
                                     p(d["zone"]), p(s["pos"]), p(s["vel"]), p(s["rho"]), p(s["p"]),
                                     p(s["type"]), p(s["zone"]), p(h), p(idx), p(cs), p(ce), self.n))

    def recover(self, d, s, idx):
        p = self._p
        self._ok(self.L.refh_recover(p(d["pos"]), p(d["vel"]), p(d["rho"]), p(d["p"]), self.n,
                                     p(idx), p(d["type"]), p(d["zone"]), p(s["pos"]), p(s["vel"]),
                                     p(s["rho"]), p(s["p"]), p(s["type"]), p(s["zone"])))

    def ns(self, s, r, cs, ce, h):
        p = self._p
        self._ok(self.L.refh_ns(p(s["pos"]), p(s["vel"]), p(s["rho"]), p(s["p"]), p(s["type"]),
                                p(r["rho_dt"]), p(r["vel_dt"]), p(cs), p(ce), self.n, p(h),
                                p(r["dofv"]), p(r["rhop_sum"]), p(r["w_sum"])))

    def pc(self, half, s, r, idx, tmp):
        p = self._p
        fn = self.L.refh_pc_prediction if half == 0 else self.L.refh_pc_correction
        self._ok(fn(p(s["pos"]), p(s["vel"]), p(s["rho"]), p(s["p"]), p(r["rho_dt"]), p(r["vel_dt"]),
                    p(idx), p(tmp["pos"]), p(tmp["vel"]), p(tmp["rho"]), self.n, p(s["type"])))

    def sync(self):
        self._ok(self.L.refh_sync())

    # whole step loop -------------------------------------------------------------
    def alloc(self, st: dict, cuda):
        import torch
        n = len(st["rho"])
        d = {k: torch.from_numpy(np.ascontiguousarray(st[k])).to(cuda)
             for k in ("pos", "vel", "rho", "p", "type")}
        d["zone"] = torch.zeros(n, dtype=torch.int32, device=cuda)
        s = {k: torch.empty_like(v) for k, v in d.items()}
        w = {"hash": torch.empty(n, dtype=torch.int32, device=cuda),
             "index": torch.empty(n, dtype=torch.int32, device=cuda),
             "cs": torch.empty(self.P.num_cells, dtype=torch.int32, device=cuda),
             "ce": torch.zeros(self.P.num_cells, dtype=torch.int32, device=cuda),
             "rho_dt": torch.zeros(n, device=cuda), "vel_dt": torch.zeros((n, 3), device=cuda),
             "dofv": torch.zeros(n, device=cuda), "rhop_sum": torch.zeros(n, device=cuda),
             "w_sum": torch.zeros(n, device=cuda)}
        tmp = {"pos": torch.zeros((n, 3), device=cuda), "vel": torch.zeros((n, 3), device=cuda),
               "rho": torch.zeros(n, device=cuda)}
        return d, s, w, tmp

    def step(self, d, s, w, tmp, nsteps: int = 1):
        """nsteps of the src step loop (src/sph/sph_run.cu:285-336), asynchronously."""
        for _ in range(nsteps):
            for half in (0, 1):
                self.calc_hash(d["pos"], w["hash"], w["index"])
                self.sort(w["hash"], w["index"])
                self.reorder(d, s, w["hash"], w["index"], w["cs"], w["ce"])
                self.ns(s, w, w["cs"], w["ce"], w["hash"])
                self.pc(half, s, w, w["index"], tmp)
                self.recover(d, s, w["index"])
