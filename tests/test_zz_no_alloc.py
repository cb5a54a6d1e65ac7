"""sph_sort_particles_noalloc: the (hash, index) sort whose scratch is a fixed device array of
the library.  Called through the C ABI and compared with sph_sort_particles (caller scratch),
which sorts the same way, on two calls in a row; sizes above SPH_SORT_NOALLOC_MAX_N are
refused before anything runs.  The file is named to be collected last, and passes alone too."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

MAX_N = 1 << 20  # SPH_SORT_NOALLOC_MAX_N


def _stream():
    import torch
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _sort_with_scratch(lib, keys, vals, key_bits):
    import torch
    from tmp_sph_gb300 import api
    h, v = keys.clone(), vals.clone()
    n = h.numel()
    scratch = torch.empty(api.sort_scratch_bytes(n), dtype=torch.uint8, device=h.device)
    st = lib.sph_sort_particles(h.data_ptr(), v.data_ptr(), n, key_bits, scratch.data_ptr(),
                                scratch.numel(), _stream())
    assert st == 0, st
    return h, v


def _sort_noalloc(lib, keys, vals, key_bits):
    h, v = keys.clone(), vals.clone()
    st = lib.sph_sort_particles_noalloc(h.data_ptr(), v.data_ptr(), h.numel(), key_bits,
                                        _stream())
    assert st == 0, st
    return h, v


def _inputs(n, seed, key_bits, device):
    import torch
    g = torch.Generator(device="cpu").manual_seed(seed)
    if key_bits == 32:
        k = torch.randint(-(1 << 31), (1 << 31) - 1, (n,), generator=g, dtype=torch.int64)
    else:
        k = torch.randint(0, 1 << key_bits, (n,), generator=g, dtype=torch.int64)
    k = k.to(torch.int32)
    return k.to(device), torch.arange(n, dtype=torch.int32).to(device)


def test_noalloc_refuses_sizes_above_its_scratch(sphlib):
    """Host-side check: n above the fixed scratch is refused with SPH_ERR_SCRATCH, and invalid
    arguments with SPH_ERR_ARG, before any CUDA call (runs without a GPU)."""
    from tmp_sph_gb300 import api
    lib = api.lib()
    buf = (C.c_int * 4)()
    assert lib.sph_sort_particles_noalloc(buf, buf, MAX_N + 1, 32, None) == api.SPH_ERR_SCRATCH
    assert lib.sph_sort_particles_noalloc(None, None, 16, 32, None) == api.SPH_ERR_ARG
    assert lib.sph_sort_particles_noalloc(buf, buf, 4, 0, None) == api.SPH_ERR_ARG
    assert lib.sph_sort_particles_noalloc(buf, buf, -1, 32, None) == api.SPH_ERR_ARG
    assert lib.sph_sort_particles_noalloc(None, None, 0, 32, None) == 0


@pytest.mark.gpu
@pytest.mark.parametrize("n,key_bits", [(300_001, 20), (200_000, 32), (MAX_N, 24)])
def test_noalloc_matches_scratch_sort_twice(sphlib, cuda, n, key_bits):
    """Two calls in a row, each on new keys, give the same (hash, index) arrays as the
    caller-scratch sort (integer sort: equality is the tolerance), and the second call changes
    no device memory figure (it allocates nothing)."""
    import torch
    from tmp_sph_gb300 import api
    lib = api.lib()
    for call in range(2):
        keys, vals = _inputs(n, seed=11 + call, key_bits=key_bits, device=cuda)
        ref_h, ref_v = _sort_with_scratch(lib, keys, vals, key_bits)
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info()[0]
        h, v = _sort_noalloc(lib, keys, vals, key_bits)
        torch.cuda.synchronize()
        free1 = torch.cuda.mem_get_info()[0]
        assert torch.equal(h, ref_h), call
        assert torch.equal(v, ref_v), call
        if call == 1:
            assert free1 == free0
    hk = h.cpu().numpy()
    assert (np.diff(hk.astype(np.int64)) >= 0).all()
    # stable: equal keys keep ascending original indices
    vv = v.cpu().numpy()
    same = np.diff(hk) == 0
    assert (np.diff(vv)[same] > 0).all()


@pytest.mark.gpu
def test_noalloc_rejects_oversize_on_device_buffers(sphlib, cuda):
    """MAX_N + 1 real device pairs: refused, and the arrays are left as they were."""
    import torch
    from tmp_sph_gb300 import api
    lib = api.lib()
    keys, vals = _inputs(MAX_N + 1, seed=5, key_bits=16, device=cuda)
    h, v = keys.clone(), vals.clone()
    st = lib.sph_sort_particles_noalloc(h.data_ptr(), v.data_ptr(), h.numel(), 16, _stream())
    torch.cuda.synchronize()
    assert st == api.SPH_ERR_SCRATCH
    assert torch.equal(h, keys) and torch.equal(v, vals)
