"""The C-ABI libraries load on a CPU host and export every declared symbol."""

import ctypes
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
HEADER = ROOT / "include" / "icsfoam_gb300.h"


def declared():
    txt = HEADER.read_text()
    names = re.findall(r"^\s*(?:int|void)\s+(ics_\w+)\s*\(", txt, flags=re.M)
    assert names, "no declarations found"
    return names


@pytest.fixture(scope="module")
def gpu_lib():
    from icsfoam_gb300 import _build

    return ctypes.CDLL(_build.build_gpu())


def test_cuda_library_exports_all_declarations(gpu_lib):
    for name in declared():
        assert hasattr(gpu_lib, name), name


def test_binding_covers_header():
    from icsfoam_gb300 import abi

    names = {n[len("ics_"):] for n in declared()}
    assert names == set(abi.EXPORTED) | {"default_config"}


def test_oracle_exports_core_api(oracle_binding):
    from icsfoam_gb300 import abi

    for name in abi._FUNCS:
        assert name in oracle_binding.fn


def test_default_configs_agree(oracle_binding, gpu_lib):
    from icsfoam_gb300 import abi

    g = abi.Config()
    gpu_lib.ics_default_config(ctypes.byref(g))
    o = oracle_binding.default_config()
    for field, _ in abi.Config._fields_:
        assert getattr(g, field) == getattr(o, field), field


def test_host_mesh_library_loads():
    from icsfoam_gb300 import ordering

    lib = ordering.host_lib()
    assert lib.ics_mesh_greedy_colour and lib.ics_mesh_rcm


def test_gpu_binding_requires_built_library(monkeypatch, tmp_path):
    """No silent fallback: a missing CUDA library is an error."""
    from icsfoam_gb300 import gpu

    monkeypatch.setattr(gpu, "_BINDING", None)
    monkeypatch.setattr(gpu, "library_path", lambda: str(tmp_path / "missing.so"))
    with pytest.raises(RuntimeError):
        gpu.binding()


def test_cuda_library_has_no_unresolved_symbols_of_its_own():
    """Every symbol the library needs comes from libc/libstdc++/libm/pthread
    (versioned) or is weak: none of our own functions is left undefined."""
    import shutil
    import subprocess

    from icsfoam_gb300 import _build

    if not shutil.which("nm"):
        pytest.skip("nm not available")
    out = subprocess.run(["nm", "-D", "--undefined-only", _build.build_gpu()], capture_output=True, text=True,
                         check=True).stdout
    bad = []
    for line in out.splitlines():
        parts = line.split()
        if len(parts) < 2 or parts[0] == "w":
            continue
        if "@" not in parts[-1]:
            bad.append(parts[-1])
    assert not bad, bad
