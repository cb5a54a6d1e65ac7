"""tmp_sph_gb300 — GB300-native weakly-compressible delta-SPH hot path.

The compute lives in libsph_gb300.so (hand-written sm_103a CUDA behind the C ABI of
include/sph_gb300.h); this package binds it with ctypes.  Build with
`python -m tmp_sph_gb300.build`.
"""
from . import api, cases  # noqa: F401
from .api import lib, SphParams, SphConfig, SphDamBreak, SphRefSimParams  # noqa: F401

__all__ = ["api", "cases", "lib", "SphParams", "SphConfig", "SphDamBreak", "SphRefSimParams"]
