"""Loader for the CUDA library (libicsgpu.so) behind the C ABI.

There is no CPU fallback: if the extension is missing or cannot load, every
entry point raises.  Build it with ``icsfoam_gb300._build.build_all()`` (the
repository's ``__graft_entry__.build()`` does the same).
"""

from __future__ import annotations

import ctypes
import os

from . import _build, abi

_BINDING = None


def library_path() -> str:
    return _build.GPU_LIB


def binding() -> abi.Binding:
    global _BINDING
    if _BINDING is None:
        path = library_path()
        if not os.path.exists(path):
            raise RuntimeError("CUDA extension %s is not built; run icsfoam_gb300._build.build_all()" % path)
        _BINDING = abi.Binding(ctypes.CDLL(path), "ics_")
    return _BINDING


def open_case(mesh, cfg) -> abi.CaseHandle:
    return abi.CaseHandle(binding(), mesh, cfg)
