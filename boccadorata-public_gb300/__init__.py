"""GB300-native (sm_103a) Sigma(2) -> Lanczos -> Dyson chain of BoccaDorata.

The compute path is the CUDA library ``libbd_gb300.so`` built from ``csrc/``;
``bd`` binds its C ABI (``include/bd_gb300.h``) and ``synth`` generates seeded
synthetic inputs in the reference's formats.
"""
from . import synth  # noqa: F401

__all__ = ["synth", "bd"]


def __getattr__(name):
    if name == "bd":
        from . import bd
        return bd
    raise AttributeError(name)
