"""Python handles over the C ABI: the resident Solver and the drop-in functions.

Device buffers are torch CUDA tensors (torch is used for device memory and streams only);
every computation happens in libsph_gb300.so.  Each drop-in function takes the same
arguments, in the same order and meaning, as the reference host function it mirrors.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import api
from .api import call, ptr


def _stream(stream) -> int | None:
    if stream is None:
        import torch
        return torch.cuda.current_stream().cuda_stream
    return getattr(stream, "cuda_stream", stream)


class Solver:
    """Resident solver context (sph_create ... sph_destroy)."""

    def __init__(self, params: api.SphParams, capacity: int | None = None,
                 precision: str = "fp32"):
        self.params = params
        cap = capacity if capacity is not None else params.num_particles
        h = C.c_void_p()
        call("sph_create", C.byref(params), cap, C.byref(h))
        self.handle = h
        self.capacity = cap
        if precision != "fp32":
            self.set_option(api.SPH_OPT_PRECISION, api.PRECISIONS[precision])

    def close(self) -> None:
        if self.handle:
            api.lib().sph_destroy(self.handle)
            self.handle = None

    __del__ = close

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def set_params(self, p: api.SphParams) -> None:
        call("sph_set_params", self.handle, C.byref(p))
        self.params = p

    def set_option(self, opt: int, value: int) -> None:
        call("sph_ctx_set_option", self.handle, opt, int(value))

    def get_option(self, opt: int) -> int:
        v = C.c_int(0)
        call("sph_ctx_get_option", self.handle, opt, C.byref(v))
        return v.value

    def upload(self, pos, vel, rho, p, typ, stream=None) -> None:
        """Host numpy arrays or device torch tensors, original particle order."""
        host = isinstance(pos, np.ndarray)
        n = len(rho)
        if host:
            pos, vel = np.ascontiguousarray(pos, np.float32), np.ascontiguousarray(vel, np.float32)
            rho, p = np.ascontiguousarray(rho, np.float32), np.ascontiguousarray(p, np.float32)
            typ = np.ascontiguousarray(typ, np.int32)
        call("sph_upload", self.handle, ptr(pos), ptr(vel), ptr(rho), ptr(p), ptr(typ), n,
             1 if host else 0, _stream(stream))
        if host:
            import torch
            torch.cuda.synchronize()
        self.n = n

    def upload_instances(self, states: list, stream=None) -> np.ndarray:
        """Upload several independent simulations (host state dicts sharing this solver's
        parameters); returns the particle offsets of the instances."""
        import torch
        counts = [len(s["rho"]) for s in states]
        off = np.zeros(len(states) + 1, np.int32)
        off[1:] = np.cumsum(counts)
        cat = {k: np.ascontiguousarray(np.concatenate([s[k] for s in states]),
                                       np.int32 if k == "type" else np.float32)
               for k in ("pos", "vel", "rho", "p", "type")}
        n = int(off[-1])
        call("sph_upload_instances", self.handle, ptr(cat["pos"]), ptr(cat["vel"]),
             ptr(cat["rho"]), ptr(cat["p"]), ptr(cat["type"]), ptr(off), len(states), n, 1,
             _stream(stream))
        torch.cuda.synchronize()
        self.n = n
        return off

    def step(self, nsteps: int = 1, stream=None) -> None:
        call("sph_step", self.handle, nsteps, _stream(stream))

    def download_device(self, out: dict, stream=None) -> None:
        call("sph_download", self.handle, ptr(out.get("pos")), ptr(out.get("vel")),
             ptr(out.get("rho")), ptr(out.get("p")), ptr(out.get("type")), 0, _stream(stream))

    def download(self, stream=None) -> dict:
        """State in original order as host numpy arrays (synchronises)."""
        import torch
        n = self.n
        out = {"pos": np.zeros((n, 3), np.float32), "vel": np.zeros((n, 3), np.float32),
               "rho": np.zeros(n, np.float32), "p": np.zeros(n, np.float32),
               "type": np.zeros(n, np.int32)}
        call("sph_download", self.handle, ptr(out["pos"]), ptr(out["vel"]), ptr(out["rho"]),
             ptr(out["p"]), ptr(out["type"]), 1, _stream(stream))
        torch.cuda.synchronize()
        return out

    def download_f64(self, stream=None) -> dict:
        """State in original order as host float64 arrays, in the solver's full precision
        (synchronises)."""
        import torch
        n = self.n
        out = {"pos": np.zeros((n, 3)), "vel": np.zeros((n, 3)), "rho": np.zeros(n),
               "p": np.zeros(n)}
        call("sph_download_f64", self.handle, ptr(out["pos"]), ptr(out["vel"]), ptr(out["rho"]),
             ptr(out["p"]), 1, _stream(stream))
        torch.cuda.synchronize()
        return out

    def step_host(self, st: dict, nsteps: int, stream=None) -> None:
        """End-to-end call with host buffers: upload, nsteps steps, download in place."""
        call("sph_step_host", self.handle, ptr(st["pos"]), ptr(st["vel"]), ptr(st["rho"]),
             ptr(st["p"]), ptr(st["type"]), len(st["rho"]), nsteps, _stream(stream))

    def error_flags(self, stream=None) -> int:
        f = C.c_uint(0)
        call("sph_read_error_flags", self.handle, C.byref(f), _stream(stream))
        return f.value

    def steps_taken(self) -> int:
        s = C.c_longlong(0)
        call("sph_steps_taken", self.handle, C.byref(s))
        return s.value

    def profile(self, reset: bool = True) -> dict:
        ms = (C.c_double * api.SPH_PHASE_COUNT)()
        ln = (C.c_longlong * api.SPH_PHASE_COUNT)()
        call("sph_profile_read", self.handle, ms, ln, 1 if reset else 0)
        return {name: {"ms": ms[i], "launches": ln[i]} for i, name in enumerate(api.PHASE_NAMES)}

    def sorted_view(self) -> tuple[int, int, int, int]:
        """(cell_start, sorted_id, sorted_hash) device addresses and the solver's cell count."""
        cs, sid, sh, nc = C.c_void_p(), C.c_void_p(), C.c_void_p(), C.c_int(0)
        call("sph_ctx_sorted_view", self.handle, C.byref(cs), C.byref(sid), C.byref(sh),
             C.byref(nc))
        return cs.value, sid.value, sh.value, nc.value

    def rebuild_count(self, stream=None) -> int:
        """Cell-list / neighbour-list rebuilds since the last upload."""
        v = C.c_uint(0)
        call("sph_read_rebuild_count", self.handle, C.byref(v), _stream(stream))
        return v.value

    def instance_rebuild_counts(self, n: int, stream=None) -> np.ndarray:
        """List rebuilds of each of the first n instances of a batch since the upload."""
        out = np.zeros(n, np.uint32)
        call("sph_read_instance_rebuild_counts", self.handle, ptr(out), n, _stream(stream))
        return out

    def list_skin(self, stream=None) -> float:
        """Skin of the current neighbour lists, as a fraction of kh."""
        v = C.c_float(0)
        call("sph_read_list_skin", self.handle, C.byref(v), _stream(stream))
        return v.value

    def probe(self, probes=(), cfl: float = 0.25, stream=None) -> tuple[list, dict]:
        """Probe values (one per (kind, x, y, z, radius, zmax) tuple or api.SphProbe) and the
        FP64 fluid statistics, computed on the GPU (synchronises)."""
        arr = (api.SphProbe * max(1, len(probes)))()
        for i, pb in enumerate(probes):
            arr[i] = pb if isinstance(pb, api.SphProbe) else api.SphProbe(*pb)
        vals = (C.c_double * max(1, len(probes)))()
        st = api.SphStats()
        call("sph_probe_read", self.handle, arr, len(probes), vals, cfl, C.byref(st),
             _stream(stream))
        return [vals[i] for i in range(len(probes))], st.as_dict()

    def ns(self, s_pos, s_vel, s_rho, s_p, s_type, rho_dt, vel_dt, cell_start, cell_end, n,
           hash_, dofv, rhop_sum=None, w_sum=None, stream=None) -> None:
        """SPH_NS_simpleversion (src/header/ns.cuh:4) on this context's parameters."""
        call("sph_ns", self.handle, ptr(s_pos), ptr(s_vel), ptr(s_rho), ptr(s_p), ptr(s_type),
             ptr(rho_dt), ptr(vel_dt), ptr(cell_start), ptr(cell_end), n, ptr(hash_), ptr(dofv),
             ptr(rhop_sum), ptr(w_sum), _stream(stream))


# ---------------------------------------------------------------- drop-in functions
def calc_hash(params, pos, hash_, index, n, stream=None) -> None:
    """calcHash (src/header/mesh.cuh:20)."""
    call("sph_calc_hash", C.byref(params), ptr(pos), ptr(hash_), ptr(index), n, _stream(stream))


def sort_particles(hash_, index, n, key_bits=32, scratch=None, stream=None) -> None:
    """sortParticles (src/header/mesh.cuh:23); scratch is a torch uint8 CUDA tensor."""
    import torch
    need = api.sort_scratch_bytes(n)
    if scratch is None or scratch.numel() < need:
        scratch = torch.empty(need, dtype=torch.uint8, device=hash_.device)
    call("sph_sort_particles", ptr(hash_), ptr(index), n, key_bits, ptr(scratch),
         scratch.numel(), _stream(stream))


def reorder(params, old_pos, old_vel, old_rho, old_p, old_type, old_zone, s_pos, s_vel, s_rho,
            s_p, s_type, s_zone, hash_, index, cell_start, cell_end, n, stream=None) -> None:
    """reorder (src/header/mesh.cuh:29)."""
    call("sph_reorder", C.byref(params), ptr(old_pos), ptr(old_vel), ptr(old_rho), ptr(old_p),
         ptr(old_type), ptr(old_zone), ptr(s_pos), ptr(s_vel), ptr(s_rho), ptr(s_p), ptr(s_type),
         ptr(s_zone), ptr(hash_), ptr(index), ptr(cell_start), ptr(cell_end), n, _stream(stream))


def recover(pos, vel, rho, p, n, index, typ, zone, s_pos, s_vel, s_rho, s_p, s_type, s_zone,
            stream=None) -> None:
    """recover (src/header/mesh.cuh:33)."""
    call("sph_recover", ptr(pos), ptr(vel), ptr(rho), ptr(p), n, ptr(index), ptr(typ), ptr(zone),
         ptr(s_pos), ptr(s_vel), ptr(s_rho), ptr(s_p), ptr(s_type), ptr(s_zone), _stream(stream))


def pc_prediction(params, s_pos, s_vel, s_rho, s_p, rho_dt, vel_dt, index, pos_tmp, vel_tmp,
                  rho_tmp, n, s_type, stream=None) -> None:
    """PC_prediction (src/header/sph.cuh:26)."""
    call("sph_pc_prediction", C.byref(params), ptr(s_pos), ptr(s_vel), ptr(s_rho), ptr(s_p),
         ptr(rho_dt), ptr(vel_dt), ptr(index), ptr(pos_tmp), ptr(vel_tmp), ptr(rho_tmp), n,
         ptr(s_type), _stream(stream))


def pc_correction(params, s_pos, s_vel, s_rho, s_p, rho_dt, vel_dt, index, pos_tmp, vel_tmp,
                  rho_tmp, n, s_type, stream=None) -> None:
    """PC_correction (src/header/sph.cuh:28)."""
    call("sph_pc_correction", C.byref(params), ptr(s_pos), ptr(s_vel), ptr(s_rho), ptr(s_p),
         ptr(rho_dt), ptr(vel_dt), ptr(index), ptr(pos_tmp), ptr(vel_tmp), ptr(rho_tmp), n,
         ptr(s_type), _stream(stream))
