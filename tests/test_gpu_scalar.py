"""Passive scalar transport on the CUDA path: known answer and oracle parity."""

import numpy as np
import pytest

from icsfoam_gb300 import abi, cases

from test_gpu_parity import perturb  # noqa: E402
from test_scalar import U0, open_channel  # noqa: E402

pytestmark = pytest.mark.gpu


def test_gpu_dual_time_steps_reproduce_implicit_upwind(gpu_binding):
    n, dt = 40, 2.0e-3
    hd, mesh, h = open_channel(gpu_binding, n, ddt_scheme=1, delta_t=dt)
    fixed = np.array([p.name == "inlet" for p in mesh.patches], np.int32)
    hd.scalar_enable(np.zeros(mesh.n_cells), fixed, np.where(fixed, 1.0, 0.0))
    order = np.argsort(mesh.C[:, 0])
    s_ref = np.zeros(n)
    c = U0 * dt / h
    A = np.diag(np.full(n, 1.0 + c)) + np.diag(np.full(n - 1, -c), -1)
    for _ in range(4):
        hd.begin_time_step()
        hd.scalar_transport(30)
        rhs = s_ref.copy()
        rhs[0] += c
        s_ref = np.linalg.solve(A, rhs)
    s, _ = hd.get_scalar()
    assert np.abs(s[order] - s_ref).max() < 1e-12


def _scalar_case(w, b, recon, D=0.0, **over):
    h = abi.CaseHandle(b, w.mesh, cases.make_config(b, w.settings, **over))
    h.set_primitive(w.p, w.U, w.T)
    P = len(w.mesh.patches)
    fixed = np.array([p.kind in (3, 5) for p in w.mesh.patches], np.int32)  # fixed / total inlet
    x = w.mesh.C[:, 0]
    s0 = 0.5 + 0.4 * np.sin(3.0 * x) * np.cos(2.0 * w.mesh.C[:, 1])
    h.scalar_enable(s0, fixed, np.where(fixed, 0.9, 0.0), D=D, recon=recon)
    return h


@pytest.mark.parametrize("name,recon,over", [
    ("bump_levels", 3, {}),
    ("bump_levels", 1, dict(ddt_scheme=2, delta_t=1e-4)),
    ("box_viscous", 4, {}),
])
def test_scalar_parity_with_oracle(gpu_binding, oracle_binding, name, recon, over):
    if name == "bump_levels":
        w = cases.bump_channel(32, 16, 10, ordering_mode="colour", flux="HLLC")
    else:
        w = perturb(cases.random_box(6))
    hs = [_scalar_case(w, b, recon, D=2e-5, **over) for b in (gpu_binding, oracle_binding)]
    for h in hs:
        if over.get("ddt_scheme"):
            h.begin_time_step()
        h.pseudo_iteration()
        h.pseudo_iteration()
    pg = hs[0].scalar_transport(3)
    po = hs[1].scalar_transport(3)
    assert pg.n_iterations == po.n_iterations
    sg, rg = hs[0].get_scalar()
    so, ro = hs[1].get_scalar()
    assert np.abs(sg - so).max() < 1e-10 * np.abs(so).max()
    assert np.abs(rg - ro).max() < 1e-10 * np.abs(ro).max()
