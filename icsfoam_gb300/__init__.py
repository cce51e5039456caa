"""GB300-native implicit coupled pseudo-time solver (ICSFoam hot path).

The product is ``libicsgpu.so`` (CUDA, sm_103a) behind the C ABI declared in
``include/icsfoam_gb300.h``.  This package holds the host-side mirror of the
reference's plugin interface (``schemes``), mesh generation and ordering,
and the ctypes binding.
"""

from . import abi, mesh, cases, ordering  # noqa: F401

__all__ = ["abi", "mesh", "cases", "ordering", "gpu"]
