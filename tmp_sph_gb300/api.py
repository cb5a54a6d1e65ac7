"""ctypes binding of the C ABI declared in include/sph_gb300.h.

The product is the CUDA library libsph_gb300.so; this module only loads it and describes
its functions and structs.  Loading fails loudly when the library has not been built: there
is no Python or CPU fallback for any operation.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libsph_gb300.so")

SPH_OK = 0
SPH_ERR_ARG = -1
SPH_ERR_CUDA = -2
SPH_ERR_NOMEM = -3
SPH_ERR_DEVICE = -4
SPH_ERR_STATE = -5
SPH_ERR_SCRATCH = -6

SPH_FLAG_OUT_OF_GRID = 0x1
SPH_FLAG_KEY_RANGE = 0x2
SPH_FLAG_NONFINITE = 0x4

SPH_EOS_LINEAR = 0
SPH_EOS_TAIT = 1

SPH_TYPE_WALL = 0
SPH_TYPE_FLUID = 1
SPH_TYPE_RIGID = 2

SPH_OPT_USE_GRAPH = 1
SPH_OPT_WALL_RATES = 2
SPH_OPT_PROFILE = 3
SPH_OPT_NEIGHBOR_LIST = 4
SPH_OPT_NEIGHBOR_CAP = 5
SPH_OPT_SKIN_PERMILLE = 6
SPH_OPT_CONDITIONAL_GRAPH = 7
SPH_OPT_PRECISION = 8
SPH_OPT_BLOCK_THREADS = 9
SPH_OPT_PARTICLES_PER_THREAD = 10
SPH_OPT_LANES_PER_PARTICLE = 12
SPH_OPT_PASS1_LANES = 14
SPH_OPT_ADAPTIVE_SKIN = 13
SPH_OPT_CELL_DIVISIONS = 16
SPH_OPT_INSTANCE_DECISIONS = 17
SPH_PREC_FP32, SPH_PREC_FP64, SPH_PREC_MIXED, SPH_PREC_MIXED_COMP = 0, 1, 2, 3
SPH_PREC_MIXED_ABS = 4
PRECISIONS = {"fp32": SPH_PREC_FP32, "fp64": SPH_PREC_FP64, "mixed": SPH_PREC_MIXED,
              "mixed_comp": SPH_PREC_MIXED_COMP, "mixed_abs": SPH_PREC_MIXED_ABS}
SPH_FLAG_NEIGHBOR_OVERFLOW = 0x8
SPH_PHASE_COUNT = 5
PHASE_NAMES = ("sort", "gather_cells", "nbr_build", "pass1", "pass2_integrate")

F3 = C.c_float * 3
I3 = C.c_int * 3


class SphParams(C.Structure):
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


class SphConfig(C.Structure):
    _fields_ = [
        ("dx", C.c_float), ("h_factor", C.c_double), ("rho0", C.c_float), ("cs", C.c_float),
        ("gravity", C.c_float), ("delta", C.c_float), ("alpha", C.c_float), ("dt", C.c_float),
        ("cfl", C.c_float), ("eos", C.c_int), ("tait_gamma", C.c_float),
        ("domain_min", F3), ("domain_max", F3), ("pad", C.c_double),
        ("cell_factor", C.c_double), ("escape_min", F3), ("escape_max", F3),
        ("escape_park", F3), ("num_particles", C.c_int), ("num_boundary", C.c_int),
        ("clamp_density", C.c_int),
    ]


class SphRefSimParams(C.Structure):
    _fields_ = (
        [("timeStep", C.c_float), ("time", C.c_float), ("numParticles", C.c_int),
         ("boundary_p_num", C.c_int), ("gravity", C.c_float)]
        + [(n, C.c_float) for n in ("gridSize", "gridxmin", "gridymin", "gridzmin", "gridxmax",
                                    "gridymax", "gridzmax")]
        + [(n, C.c_int) for n in ("gridxdim", "gridydim", "gridzdim", "numCells", "hash_max",
                                  "hash_min")]
        + [(n, C.c_float) for n in ("pre_set_domain_x_min", "pre_set_domain_x_max",
                                    "pre_set_domain_y_min", "pre_set_domain_y_max",
                                    "pre_set_domain_z_min", "pre_set_domain_z_max", "particleR",
                                    "h", "kh", "eta", "delta", "afa", "SpikyKern", "LapKern",
                                    "Poly6Kern", "minDist", "particleMass", "restDensity",
                                    "viscosity", "stiffness", "cs", "adh", "namuta_threshold_1",
                                    "namuta_threshold_2", "CFL", "Ma", "conc_0", "conc_t",
                                    "PST_R", "PST_n", "w_deltar")]
        + [(n, C.c_int) for n in ("ngp", "nnode", "n_edge", "num_vp", "max_nspnode", "nele")]
        + [("mat_para", F3)]
    )


class SphDamBreak(C.Structure):
    _fields_ = [
        ("dx", C.c_float), ("tank", F3), ("block", F3), ("wall_layers", C.c_int),
        ("has_obstacle", C.c_int), ("obstacle_min", F3), ("obstacle_max", F3),
        ("jitter", C.c_float), ("seed", C.c_ulonglong), ("hydrostatic", C.c_int),
        ("rho0", C.c_float), ("gravity", C.c_float), ("cs", C.c_float), ("eos", C.c_int),
        ("tait_gamma", C.c_float),
    ]


SPH_MAX_INSTANCES = 4096
SPH_PROBE_PRESSURE, SPH_PROBE_HEIGHT, SPH_PROBE_FRONT = 0, 1, 2
SPH_MAX_PROBES = 32


class SphProbe(C.Structure):
    _fields_ = [("kind", C.c_int), ("x", C.c_float), ("y", C.c_float), ("z", C.c_float),
                ("radius", C.c_float), ("zmax", C.c_float)]


class SphStats(C.Structure):
    _fields_ = [("fluid", C.c_longlong), ("parked", C.c_longlong), ("mass", C.c_double),
                ("kinetic", C.c_double), ("potential", C.c_double), ("max_speed", C.c_double),
                ("rho_min", C.c_double), ("rho_max", C.c_double), ("front_x", C.c_double),
                ("cfl_dt", C.c_double)]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


_P = C.c_void_p
_I = C.c_int
_PP = C.POINTER(SphParams)

# name -> (restype, argtypes)
_PROTOS = {
    "sph_params_derive": (_I, [C.POINTER(SphConfig), _PP]),
    "sph_params_reference": (_I, [C.c_float, C.c_float, C.c_float, C.c_float, _I, _I, _PP]),
    "sph_params_from_reference": (_I, [C.POINTER(SphRefSimParams), _PP]),
    "sph_params_to_reference": (_I, [_PP, C.POINTER(SphRefSimParams)]),
    "sph_status_string": (C.c_char_p, [_I]),
    "sph_version": (C.c_char_p, []),
    "sph_measure_fp32_peak": (_I, [_P, _I, _I, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                   _P]),
    "sph_calc_hash": (_I, [_PP, _P, _P, _P, _I, _P]),
    "sph_sort_scratch_bytes": (_I, [_I, C.POINTER(C.c_size_t)]),
    "sph_sort_particles": (_I, [_P, _P, _I, _I, _P, C.c_size_t, _P]),
    "sph_sort_particles_noalloc": (_I, [_P, _P, _I, _I, _P]),
    "sph_reorder": (_I, [_PP] + [_P] * 16 + [_I, _P]),
    "sph_recover": (_I, [_P, _P, _P, _P, _I, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P]),
    "sph_pc_prediction": (_I, [_PP] + [_P] * 10 + [_I, _P, _P]),
    "sph_pc_correction": (_I, [_PP] + [_P] * 10 + [_I, _P, _P]),
    "sph_create": (_I, [_PP, _I, C.POINTER(_P)]),
    "sph_destroy": (_I, [_P]),
    "sph_set_params": (_I, [_P, _PP]),
    "sph_get_params": (_I, [_P, _PP]),
    "sph_ctx_set_option": (_I, [_P, _I, _I]),
    "sph_ctx_get_option": (_I, [_P, _I, _P]),
    "sph_ns": (_I, [_P] + [_P] * 9 + [_I] + [_P] * 4 + [_P]),
    "sph_upload": (_I, [_P, _P, _P, _P, _P, _P, _I, _I, _P]),
    "sph_upload_instances": (_I, [_P, _P, _P, _P, _P, _P, _P, _I, _I, _I, _P]),
    "sph_instances": (_I, [_P, C.POINTER(_I)]),
    "sph_download": (_I, [_P, _P, _P, _P, _P, _P, _I, _P]),
    "sph_download_f64": (_I, [_P, _P, _P, _P, _P, _I, _P]),
    "sph_step": (_I, [_P, _I, _P]),
    "sph_step_host": (_I, [_P, _P, _P, _P, _P, _P, _I, _I, _P]),
    "sph_ctx_sorted_view": (_I, [_P, C.POINTER(_P), C.POINTER(_P), C.POINTER(_P), C.POINTER(_I)]),
    "sph_read_rebuild_count": (_I, [_P, C.POINTER(C.c_uint), _P]),
    "sph_read_instance_rebuild_counts": (_I, [_P, _P, _I, _P]),
    "sph_read_list_skin": (_I, [_P, C.POINTER(C.c_float), _P]),
    "sph_snapshot_begin": (_I, [_P, _P, _P, _P, _P, _P, _P]),
    "sph_snapshot_wait": (_I, [_P]),
    "sph_snapshot_query": (_I, [_P, C.POINTER(_I)]),
    "sph_write_vtk": (_I, [C.c_char_p, _I, _P, _P, _P, _P, _I]),
    "sph_probe_read": (_I, [_P, C.POINTER(SphProbe), _I, C.POINTER(C.c_double), C.c_double,
                            C.POINTER(SphStats), _P]),
    "sph_read_error_flags": (_I, [_P, C.POINTER(C.c_uint), _P]),
    "sph_steps_taken": (_I, [_P, C.POINTER(C.c_longlong)]),
    "sph_profile_read": (_I, [_P, C.POINTER(C.c_double), C.POINTER(C.c_longlong), _I]),
    "sph_shim_set_reference_params": (_I, [C.POINTER(SphRefSimParams)]),
    "sph_shim_set_params": (_I, [_PP]),
    "sph_shim_release": (_I, []),
    "sph_dam_break_count": (_I, [C.POINTER(SphDamBreak), C.POINTER(_I), C.POINTER(_I)]),
    "sph_dam_break_generate": (_I, [C.POINTER(SphDamBreak), _P, _P, _P, _P, _P, _I]),
    "sph_write_dat": (_I, [C.c_char_p, _P, _P, _P, _P, _P, _I]),
    "sph_read_dat": (_I, [C.c_char_p, _P, _P, _P, _P, _P, _P, _P, _I]),
}

# Functions of include/sph_gb300.h that the library must export (checked by the CPU tests).
EXPORTED = sorted(_PROTOS)

_lib = None


class SphError(RuntimeError):
    def __init__(self, fn: str, status: int):
        super().__init__(f"{fn}: {status_string(status)} ({status})")
        self.status = status


def lib() -> C.CDLL:
    """The loaded CUDA library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(
                f"{LIB_PATH} is missing: build it with `python -m tmp_sph_gb300.build` "
                "(there is no CPU fallback)")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in _PROTOS.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def status_string(st: int) -> str:
    return lib().sph_status_string(st).decode()


def check(fn: str, st: int) -> None:
    if st != SPH_OK:
        raise SphError(fn, st)


def call(name: str, *args) -> None:
    check(name, getattr(lib(), name)(*args))


def ptr(x) -> int | None:
    """Device/host address of a torch tensor or numpy array (None for None)."""
    if x is None:
        return None
    if isinstance(x, np.ndarray):
        assert x.flags["C_CONTIGUOUS"]
        return x.ctypes.data
    assert x.is_contiguous()
    return x.data_ptr()


# ---------------------------------------------------------------- parameters
def params_reference(dx: float, vlx: float, vly: float, vlz: float, np_: int = 0,
                     nb: int = 0) -> SphParams:
    p = SphParams()
    call("sph_params_reference", dx, vlx, vly, vlz, np_, nb, C.byref(p))
    return p


def params_derive(cfg: SphConfig) -> SphParams:
    p = SphParams()
    call("sph_params_derive", C.byref(cfg), C.byref(p))
    return p


def params_from_reference(r: SphRefSimParams) -> SphParams:
    p = SphParams()
    call("sph_params_from_reference", C.byref(r), C.byref(p))
    return p


def params_to_reference(p: SphParams) -> SphRefSimParams:
    r = SphRefSimParams()
    call("sph_params_to_reference", C.byref(p), C.byref(r))
    return r


def sort_scratch_bytes(n: int) -> int:
    b = C.c_size_t(0)
    call("sph_sort_scratch_bytes", n, C.byref(b))
    return b.value


# ---------------------------------------------------------------- initial conditions
def dam_break_count(d: SphDamBreak) -> tuple[int, int]:
    nf, nb = C.c_int(0), C.c_int(0)
    call("sph_dam_break_count", C.byref(d), C.byref(nf), C.byref(nb))
    return nf.value, nb.value


def dam_break_generate(d: SphDamBreak) -> dict:
    """Host arrays of a generated dam break: pos/vel (n,3) f32, rho/p (n,) f32, type (n,) i32."""
    nf, nb = dam_break_count(d)
    n = nf + nb
    pos = np.zeros((n, 3), np.float32)
    vel = np.zeros((n, 3), np.float32)
    rho = np.zeros(n, np.float32)
    p = np.zeros(n, np.float32)
    typ = np.zeros(n, np.int32)
    call("sph_dam_break_generate", C.byref(d), ptr(pos), ptr(vel), ptr(rho), ptr(p), ptr(typ), n)
    return {"pos": pos, "vel": vel, "rho": rho, "p": p, "type": typ, "n_fluid": nf,
            "n_boundary": nb}


def write_dat(directory: str, st: dict) -> None:
    call("sph_write_dat", directory.encode(), ptr(st["pos"]), ptr(st["vel"]), ptr(st["rho"]),
         ptr(st["p"]), ptr(st["type"]), len(st["rho"]))


def read_dat(directory: str, n: int) -> dict:
    out = {"pos": np.zeros((n, 3), np.float32), "vel": np.zeros((n, 3), np.float32),
           "ac": np.zeros((n, 3), np.float32), "rho": np.zeros(n, np.float32),
           "p": np.zeros(n, np.float32), "type": np.zeros(n, np.int32),
           "zone": np.zeros(n, np.int32)}
    call("sph_read_dat", directory.encode(), ptr(out["pos"]), ptr(out["vel"]), ptr(out["ac"]),
         ptr(out["rho"]), ptr(out["p"]), ptr(out["type"]), ptr(out["zone"]), n)
    return out
