"""Oracle (CPU) and CUDA path (GPU) against the committed golden vectors.

Tolerance: 1e-12 of each equation's max-norm for fluxes, the residual source
and the Jacobian action; 1e-10 for the GMRES increment, the updated state
and the three-iteration rho L2 residual history.
"""

import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

import make_golden  # noqa: E402

NAMES = sorted(make_golden.CASES)


def err(a, b):
    a = np.asarray(a, float)
    b = np.asarray(b, float)
    if b.ndim == 2 and b.shape[1] == 5:
        s = np.abs(b).max(axis=0)
        s[1:4] = s[1:4].max()
    else:
        s = np.abs(b).max(axis=0) if b.ndim else abs(b)
    s = np.where(s == 0, 1.0, s)
    return float((np.abs(a - b) / s).max())


def check(d, g):
    for k in ("phi", "phiU", "phiE", "src", "Ax"):
        assert err(d[k], g[k]) < 1e-12, k
    assert int(d["gmres_cycles"]) == int(g["gmres_cycles"])
    for k in ("dW", "W"):
        assert err(d[k], g[k]) < 1e-10, k
    assert np.allclose(d["hist"], g["hist"], rtol=1e-9, atol=0)


@pytest.mark.parametrize("name", NAMES)
def test_oracle_reproduces_golden(oracle_binding, name):
    g = np.load(os.path.join(HERE, "golden", name + ".npz"))
    check(make_golden.compute(oracle_binding, name), g)


@pytest.mark.gpu
@pytest.mark.parametrize("name", NAMES)
def test_gpu_matches_golden(gpu_binding, name):
    g = np.load(os.path.join(HERE, "golden", name + ".npz"))
    check(make_golden.compute(gpu_binding, name), g)
