"""GB300-native adaptive PBF substep (neighbour search, Jacobi incompressibility,
split/merge) behind a C ABI that mirrors the stage objects of cg-tuwien/APBF.

The compute path is the CUDA library apbf_gb300/_lib/libapbf_gb300.so (built by
apbf_gb300.build); importing the stage API loads it and fails loudly if it is
missing.  There is no CPU fallback.
"""
from . import _native  # noqa: F401

__all__ = ["_native"]
