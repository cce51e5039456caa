"""A compiled C++ caller of the C ABI (tests/cxx/ics_caller.cpp).

Every other test reaches the libraries through ctypes, which would not notice
a declaration in include/icsfoam_gb300.h drifting away from what the
libraries export.  Here a C++ translation unit includes the header, describes
a channel mesh, creates a handle and runs pseudo iterations:

* on the CPU it is compiled and linked against the CUDA library (so every
  entry point it uses must be exported with the declared signature) and, with
  the icsref_ prefix, against the oracle, which it then runs;
* on the GPU both executables run and their residual histories and final
  states agree (FP64: 1e-9 relative, the tolerance of the lockstep
  trajectory tests).
"""

import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cxx", "ics_caller.cpp")


def _compile(out, oracle):
    from icsfoam_gb300 import _build

    import oracle as oracle_pkg

    if oracle:
        libdir = os.path.dirname(oracle_pkg.build.build())
        libs = ["-DICS_CALLER_ORACLE", "-L" + libdir, "-licsref"]
    else:
        libdir = os.path.dirname(_build.GPU_LIB)
        if not os.path.exists(_build.GPU_LIB):
            pytest.skip("CUDA library not built")
        libs = ["-L" + libdir, "-licsgpu"]
    cmd = ["g++", "-O2", "-std=c++17", "-Wall", "-Wextra", "-Werror", "-I" + os.path.join(ROOT, "include"), SRC,
           "-o", out] + libs + ["-Wl,-rpath," + libdir]
    subprocess.check_call(cmd)
    return out


def _run(exe, *args):
    out = subprocess.run([exe] + [str(a) for a in args], check=True, capture_output=True, text=True).stdout
    rows = [line.split() for line in out.splitlines()]
    hist = np.array([[float(r[3]), float(r[5])] for r in rows if r[0] == "iter"])
    sumW = np.array([float(v) for v in rows[-1][1:]])
    return hist, sumW


def test_cxx_caller_compiles_links_and_runs_on_the_oracle(tmp_path):
    _compile(str(tmp_path / "caller_gpu"), oracle=False)
    exe = _compile(str(tmp_path / "caller_ref"), oracle=True)
    hist, sumW = _run(exe, 24, 8, 4, 4, 0)
    assert hist.shape == (4, 2)
    assert np.all(np.isfinite(hist)) and np.all(hist[:, 0] > 0) and np.all(hist[:, 1] >= 1)
    assert np.all(np.isfinite(sumW)) and sumW[0] > 0 and sumW[4] > 0


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [0, 1])
def test_cxx_caller_gpu_matches_oracle(tmp_path, precision):
    gpu = _compile(str(tmp_path / "caller_gpu"), oracle=False)
    ref = _compile(str(tmp_path / "caller_ref"), oracle=True)
    hg, sg = _run(gpu, 24, 8, 4, 4, precision)
    ho, so = _run(ref, 24, 8, 4, 4, 0)
    tol = 1e-9 if precision == 0 else 1e-4
    if precision == 0:
        assert np.array_equal(hg[:, 1], ho[:, 1])
    assert np.max(np.abs(hg[:, 0] - ho[:, 0]) / ho[:, 0]) < tol
    scale = np.abs(so)
    scale[1:4] = scale[1:4].max()
    assert np.max(np.abs(sg - so) / scale) < tol
