"""CPU FP64 oracle (test infrastructure only).

Loads oracle/libicsref.so, which exports the package's C ABI with the prefix
``icsref_``.  Only tests, ``__graft_entry__.smoke()`` and the CPU-baseline
legs of ``bench.py`` use it, as the checker and the timed CPU baseline.
"""

import ctypes
import os

from . import build as _build

_BINDING = None


def binding():
    global _BINDING
    if _BINDING is None:
        from icsfoam_gb300 import abi

        lib = ctypes.CDLL(_build.build())
        _BINDING = abi.Binding(lib, "icsref_")
    return _BINDING


def open_case(mesh, cfg):
    from icsfoam_gb300 import abi

    return abi.CaseHandle(binding(), mesh, cfg)
