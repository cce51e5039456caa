"""Viscous Jacobian without LaxFriedrichJacobian on the CUDA path.

The non-LF viscous blocks (laplacians of mu and alphaEff through -U/rho,
1/rho, -E/rho + |U|^2/rho; the physical patches' boundary terms; the coupled
interface at the patch value) against the oracle on the randomised viscous
box and the annular sector with its rotational cyclic pair: Jacobian blocks,
matrix action and LU-SGS in FP64, pseudo-iteration trajectories in FP64 and
mixed precision.  Tolerances as in the other parity tests.
"""

import numpy as np
import pytest

from test_gpu_parity import relerr  # noqa: E402
from test_viscous_jacobian import open_case, workload  # noqa: E402

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["box", "sector"])
def test_non_lf_jacobian_parity(gpu_binding, oracle_binding, name):
    w = workload(name)
    hg = open_case(gpu_binding, w, viscous_lf_jacobian=0)
    ho = open_case(oracle_binding, w, viscous_lf_jacobian=0)
    assert relerr(hg.residual(), ho.residual()) < 1e-12
    for h in (ho, hg):
        h.assemble_jacobian()
    Do, Lo, Uo = ho.get_jacobian()
    Dg, Lg, Ug = hg.get_jacobian()
    assert relerr(Dg, Do) < 1e-12
    assert relerr(Lg, Lo) < 1e-12
    assert relerr(Ug, Uo) < 1e-12
    x = np.random.default_rng(1).standard_normal((w.mesh.n_cells, 5))
    assert relerr(hg.matrix_mul(x), ho.matrix_mul(x)) < 1e-12
    assert relerr(hg.precondition(x), ho.precondition(x)) < 1e-12


@pytest.mark.parametrize("name,precision,tol", [("box", 0, 1e-10), ("sector", 0, 1e-10), ("box", 1, 1e-4),
                                                ("sector", 1, 1e-4)])
def test_non_lf_trajectory(gpu_binding, oracle_binding, name, precision, tol):
    w = workload(name)
    hg = open_case(gpu_binding, w, viscous_lf_jacobian=0, precision=precision)
    ho = open_case(oracle_binding, w, viscous_lf_jacobian=0)
    for it in range(3):
        sg, so = hg.pseudo_iteration(), ho.pseudo_iteration()
        assert sg.perf.n_iterations == so.perf.n_iterations or precision
        assert relerr(hg.get_state()["W"], ho.get_state()["W"]) < tol, it
