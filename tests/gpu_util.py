"""Helpers for the GPU tests: host <-> torch device copies and cases."""
from __future__ import annotations

import numpy as np


def dev(a, cuda):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).to(cuda)


def host(t) -> np.ndarray:
    import torch
    torch.cuda.synchronize()
    return t.detach().cpu().numpy()


def empty_like_np(a, cuda):
    import torch
    dt = {np.dtype(np.float32): torch.float32, np.dtype(np.int32): torch.int32}[np.dtype(a.dtype)]
    return torch.empty(a.shape, dtype=dt, device=cuda)


def perturbed(st: dict, seed: int = 3, vamp: float = 0.3, ramp: float = 0.02) -> dict:
    """Copy of a state with random fluid velocities and densities, so the neighbour sums do
    not cancel the way they do in a fluid at rest."""
    rng = np.random.default_rng(seed)
    out = {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in st.items()}
    fl = out["type"] == 1
    out["vel"][fl] = rng.uniform(-vamp, vamp, (fl.sum(), 3)).astype(np.float32)
    out["rho"][fl] = (1000.0 * (1.0 + rng.uniform(0, ramp, fl.sum()))).astype(np.float32)
    out["p"][fl] = (625.0 * (out["rho"][fl] - 1000.0)).astype(np.float32)
    return out
