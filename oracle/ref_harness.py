"""Python handle on the reference's own compiled kernels (oracle/_ref).  TEST INFRASTRUCTURE.

RefHarness(version) runs one of the reference's code trees — "src" (the baseline) or the
optimisation snapshots "v0".."v4" — on the GPU with its own launch shapes, on torch CUDA
buffers, to generate golden fixtures and to time the reference's CUDA step loops.  Needs
oracle/_ref/ref_<version>.fatbin (built where the reference sources are, see ref_build.py)
and builds the harness library itself.
"""
from __future__ import annotations

import ctypes as C
import math
import os

import numpy as np

from . import ref_build

F = C.c_float
I = C.c_int

_BASE_FIELDS = (
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


class RefSimParams(C.Structure):
    """Byte layout of the reference's SimParams (src/header/data_struct.cuh:4-44)."""
    _fields_ = _BASE_FIELDS


class RefSimParamsV4(C.Structure):
    """opt_src_v4's SimParams: five precomputed products appended
    (opt_src_v4/header/data_struct.cuh:46-50)."""
    _fields_ = _BASE_FIELDS + [(n, F) for n in ("h2", "eta2", "cs2", "delta_h_cs", "h_cs_rho_m")]


def simparams_from(P, n: int, version: str = "src"):
    """The reference's SimParams for oracle parameters P (the fields its kernels read), with
    hash_max as src/sph/sph_run.cu:92 sets it.  For v4 the grid uses gridSize = particleR
    (opt_src_v4/sph/sph_run.cu:73) and the five products of :104-109."""
    f32 = np.float32
    r = (RefSimParamsV4 if version == "v4" else RefSimParams)()
    cell = P.cell_size
    dims = [P.grid_dim[0], P.grid_dim[1], P.grid_dim[2]]
    if version == "v4":
        cell = P.dx
        dims = [int(math.ceil(float((f32(P.grid_max[c]) - f32(P.grid_min[c])) / f32(cell))))
                for c in range(3)]
    gx, gy, gz = dims
    r.timeStep, r.numParticles, r.boundary_p_num, r.gravity = P.dt, n, P.num_boundary, P.gravity
    r.gridSize = cell
    r.gridxmin, r.gridymin, r.gridzmin = P.grid_min[0], P.grid_min[1], P.grid_min[2]
    r.gridxmax, r.gridymax, r.gridzmax = P.grid_max[0], P.grid_max[1], P.grid_max[2]
    r.gridxdim, r.gridydim, r.gridzdim, r.numCells = gx, gy, gz, gx * gy * gz
    r.hash_max, r.hash_min = gx * gy * gz + gx * gy + gx, 0
    r.particleR, r.h, r.kh, r.eta, r.delta, r.afa = P.dx, P.h, P.kh, P.eta, P.delta, P.alpha
    r.particleMass, r.restDensity, r.cs, r.adh = P.mass, P.rho0, P.cs, P.adh
    if version == "v4":
        h, cs, eta = f32(P.h), f32(P.cs), f32(P.eta)
        r.h2, r.cs2, r.eta2 = float(h * h), float(cs * cs), float(eta * eta)
        r.delta_h_cs = float(f32(P.delta) * h * cs)
        r.h_cs_rho_m = float(h * cs * f32(P.rho0) * f32(P.mass))
    return r


_LIB = None


def _lib():
    global _LIB
    if _LIB is None:
        L = C.CDLL(ref_build.build_harness())
        L.refh_error.restype = C.c_char_p
        L.refh_params_bytes.restype = C.c_size_t
        L.refh_load.argtypes = [C.c_char_p]
        _LIB = L
    return _LIB


class RefHarness:
    def __init__(self, version: str = "src"):
        fat = ref_build.fatbin_path(version)
        if not os.path.exists(fat):
            raise FileNotFoundError(f"{fat} missing (built from the reference sources)")
        self.L = _lib()
        self.version = version
        h = self.L.refh_load(fat.encode())
        if h < 0:
            raise RuntimeError("reference harness: " + self.L.refh_error().decode())
        self.h = h
        self.pingpong = version != "src"  # v0..v4 drop recover for ping-pong buffers
        self.n = 0

    def _ok(self, rc):
        if rc != 0:
            raise RuntimeError(f"reference harness ({self.version}): " +
                               self.L.refh_error().decode())

    def set_params(self, P, n: int) -> None:
        r = simparams_from(P, n, self.version)
        assert self.L.refh_params_bytes(self.h) == C.sizeof(r), \
            (self.L.refh_params_bytes(self.h), C.sizeof(r))
        self._ok(self.L.refh_set_params(self.h, C.byref(r), C.c_size_t(C.sizeof(r)), r.numCells))
        self.P, self.n, self.sp = P, n, r

    # device buffers ------------------------------------------------------------
    @staticmethod
    def _p(t):
        return C.c_void_p(t.data_ptr()) if t is not None else C.c_void_p(0)

    def calc_hash(self, pos, h, idx):
        self._ok(self.L.refh_calc_hash(self.h, self._p(pos), self._p(h), self._p(idx), self.n))

    def sort(self, h, idx):
        self._ok(self.L.refh_sort(self._p(h), self._p(idx), self.n))

    def reorder(self, d, s, h, idx, cs, ce, tl=None, tr=None):
        p = self._p
        self._ok(self.L.refh_reorder(self.h, p(d["pos"]), p(d["vel"]), p(d["rho"]), p(d["p"]),
                                     p(d["type"]), p(d["zone"]), p(s["pos"]), p(s["vel"]),
                                     p(s["rho"]), p(s["p"]), p(s["type"]), p(s["zone"]), p(h),
                                     p(idx), p(cs), p(ce), self.n, p(tl), p(tr)))

    def recover(self, d, s, idx):
        p = self._p
        self._ok(self.L.refh_recover(self.h, p(d["pos"]), p(d["vel"]), p(d["rho"]), p(d["p"]),
                                     self.n, p(idx), p(d["type"]), p(d["zone"]), p(s["pos"]),
                                     p(s["vel"]), p(s["rho"]), p(s["p"]), p(s["type"]),
                                     p(s["zone"])))

    def ns(self, s, r, cs, ce, h):
        p = self._p
        self._ok(self.L.refh_ns(self.h, p(s["pos"]), p(s["vel"]), p(s["rho"]), p(s["p"]),
                                p(s["type"]), p(r["rho_dt"]), p(r["vel_dt"]), p(cs), p(ce), self.n,
                                p(h), p(r["dofv"]), p(r["rhop_sum"]), p(r["w_sum"])))

    def pc(self, half, s, r, idx, tmp):
        p = self._p
        fn = self.L.refh_pc_prediction if half == 0 else self.L.refh_pc_correction
        self._ok(fn(self.h, p(s["pos"]), p(s["vel"]), p(s["rho"]), p(s["p"]), p(r["rho_dt"]),
                    p(r["vel_dt"]), p(idx), p(tmp["pos"]), p(tmp["vel"]), p(tmp["rho"]), self.n,
                    p(s["type"])))

    def sync(self):
        self._ok(self.L.refh_sync())

    def check_in_grid(self, pos: np.ndarray) -> None:
        """Refuse inputs with a particle outside the grid: the reference's reorder stores
        cellStart[hash] with no range check (src/lib/mesh.cu:119), so such a particle would make
        it write outside the cell array.  Evaluated on the host with the float expression of
        src/lib/mesh.cu:6-17 and this version's grid."""
        r = self.sp
        f32 = np.float32
        gmin = [f32(r.gridxmin), f32(r.gridymin), f32(r.gridzmin)]
        dims = [r.gridxdim, r.gridydim, r.gridzdim]
        p = np.asarray(pos, np.float32).reshape(-1, 3)
        for c in range(3):
            g = np.floor((p[:, c] - gmin[c]) / f32(r.gridSize))
            if not (np.isfinite(g).all() and g.min() >= 0 and g.max() < dims[c]):
                raise ValueError(f"particle outside the reference grid on axis {c}: cell range "
                                 f"[{g.min()}, {g.max()}] vs [0, {dims[c]})")

    # whole step loop -------------------------------------------------------------
    def alloc(self, st: dict, cuda):
        """Device buffers for the step loop.  The cell arrays hold hash_max + 8 entries (cells
        past numCells read as empty): the reference's neighbour loops and v2's empty-cell fill
        index up to hash_max, which is larger than numCells."""
        import torch
        n = len(st["rho"])
        self.check_in_grid(st["pos"])
        d = {k: torch.from_numpy(np.ascontiguousarray(st[k])).to(cuda)
             for k in ("pos", "vel", "rho", "p", "type")}
        d["zone"] = torch.zeros(n, dtype=torch.int32, device=cuda)
        s = {k: torch.empty_like(v) for k, v in d.items()}
        ncell = self.sp.hash_max + 8
        w = {"hash": torch.empty(n, dtype=torch.int32, device=cuda),
             "index": torch.empty(n, dtype=torch.int32, device=cuda),
             "cs": torch.full((ncell,), -1, dtype=torch.int32, device=cuda),
             "ce": torch.zeros(ncell, dtype=torch.int32, device=cuda),
             "rho_dt": torch.zeros(n, device=cuda), "vel_dt": torch.zeros((n, 3), device=cuda),
             "dofv": torch.zeros(n, device=cuda), "rhop_sum": torch.zeros(n, device=cuda),
             "w_sum": torch.zeros(n, device=cuda),
             "table_l": torch.zeros(n, dtype=torch.int32, device=cuda),
             "table_r": torch.zeros(n, dtype=torch.int32, device=cuda)}
        tmp = {"pos": torch.zeros((n, 3), device=cuda), "vel": torch.zeros((n, 3), device=cuda),
               "rho": torch.zeros(n, device=cuda)}
        return d, s, w, tmp

    def step(self, d, s, w, tmp, nsteps: int = 1):
        """nsteps of the version's step loop: src/sph/sph_run.cu:285-336 (recover after each
        half step) or the ping-pong loop of opt_src_v0/sph/sph_run.cu:269-309."""
        for _ in range(nsteps):
            if not self.pingpong:
                for half in (0, 1):
                    self.calc_hash(d["pos"], w["hash"], w["index"])
                    self.sort(w["hash"], w["index"])
                    self.reorder(d, s, w["hash"], w["index"], w["cs"], w["ce"])
                    self.ns(s, w, w["cs"], w["ce"], w["hash"])
                    self.pc(half, s, w, w["index"], tmp)
                    self.recover(d, s, w["index"])
            else:
                self.calc_hash(d["pos"], w["hash"], w["index"])
                self.sort(w["hash"], w["index"])
                self.reorder(d, s, w["hash"], w["index"], w["cs"], w["ce"], w["table_l"], w["table_r"])
                self.ns(s, w, w["cs"], w["ce"], w["hash"])
                self.pc(0, s, w, w["index"], tmp)
                self.calc_hash(s["pos"], w["hash"], w["index"])
                self.sort(w["hash"], w["index"])
                self.reorder(s, d, w["hash"], w["index"], w["cs"], w["ce"], w["table_r"], w["table_l"])
                self.ns(d, w, w["cs"], w["ce"], w["hash"])
                self.pc(1, d, w, w["index"], tmp)

    def state(self, d, s):
        """Current state (x, v, rho, p, type) as host arrays in original particle order.  The
        ping-pong versions end a step in d in the order of the second sort; w['table_*'] keep the
        reference's own bookkeeping, here the order is restored by re-sorting on a particle id
        carried in the zone array (set by init_ids)."""
        out = {k: d[k].detach().cpu().numpy() for k in ("pos", "vel", "rho", "p", "type", "zone")}
        if self.pingpong:
            order = np.argsort(out["zone"], kind="stable")
            out = {k: v[order] for k, v in out.items()}
        return out

    @staticmethod
    def init_ids(d):
        """Tag particles with their original index in the (otherwise unused) zone array, which
        every version's reorder gathers along with the state."""
        import torch
        d["zone"].copy_(torch.arange(d["zone"].numel(), dtype=torch.int32, device=d["zone"].device))
