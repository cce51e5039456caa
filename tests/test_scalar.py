"""Passive scalar transport (dbnsFoam calculateScalarTransport.H) in the oracle.

Known answers: (1) in a uniform stream a uniform scalar is a fixed point;
(2) with a uniform stream the Roe flux is exact upwinding, so converged dual
time steps reproduce the implicit-Euler upwind solution of s_t + u s_x = 0
(lower bidiagonal system solved here with numpy); (3) the steady state of
advection from a fixed inlet value is that value everywhere.
"""

import numpy as np
import pytest

from icsfoam_gb300 import abi, cases
from icsfoam_gb300 import mesh as M

U0, P0, T0 = 50.0, 1.0e5, 300.0


def channel_1d(n=40, length=1.0):
    xs = np.linspace(0.0, length, n + 1)
    h = length / n
    g = np.zeros((n + 1, 2, 2, 3))
    g[..., 0] = xs[:, None, None]
    g[:, 1, :, 1] = h
    g[:, :, 1, 2] = h
    inlet = M.Patch("inlet", M.PATCH_FIXED, p=P0, T=T0, U=(U0, 0.0, 0.0))
    outlet = M.Patch("outlet", M.PATCH_ZERO_GRADIENT)
    empty = M.Patch("empty", M.PATCH_EMPTY)
    sides = {"xmin": inlet, "xmax": outlet, "ymin": empty, "ymax": empty, "zmin": empty, "zmax": empty}
    return M.hex_mesh(g, sides), h


def open_channel(b, n=40, **over):
    mesh, h = channel_1d(n)
    N = mesh.n_cells
    settings = dict(cases.thermo_settings(), flux_scheme=0, n_directions=8, max_iter=50, tolerance=1e-14,
                    rel_tol=1e-12, pseudo_tol=1e-30, pseudo_tol_rel=1e-30, pseudo_co_num=1e6,
                    pseudo_co_num_max=1e6)
    settings.update(over)
    hd = abi.CaseHandle(b, mesh, cases.make_config(b, settings))
    U = np.zeros((N, 3))
    U[:, 0] = U0
    hd.set_primitive(np.full(N, P0), U, np.full(N, T0))
    hd.residual()  # local pseudo time step of the (uniform) flow
    return hd, mesh, h


def test_uniform_scalar_in_uniform_stream_is_a_fixed_point(oracle_binding):
    hd, mesh, _ = open_channel(oracle_binding)
    P = len(mesh.patches)
    fixed = np.array([p.name == "inlet" for p in mesh.patches], np.int32)
    hd.scalar_enable(np.full(mesh.n_cells, 0.3), fixed, np.full(P, 0.3))
    perf = hd.scalar_transport(3)
    s, rs = hd.get_scalar()
    assert np.abs(s - 0.3).max() < 1e-13


def test_dual_time_steps_reproduce_implicit_upwind(oracle_binding):
    n, dt = 40, 2.0e-3
    hd, mesh, h = open_channel(oracle_binding, n, ddt_scheme=1, delta_t=dt)
    fixed = np.array([p.name == "inlet" for p in mesh.patches], np.int32)
    s0 = np.zeros(mesh.n_cells)
    hd.scalar_enable(s0, fixed, np.where(fixed, 1.0, 0.0))
    order = np.argsort(mesh.C[:, 0])  # cells along x
    s_ref = s0[order].copy()
    c = U0 * dt / h
    A = np.diag(np.full(n, 1.0 + c)) + np.diag(np.full(n - 1, -c), -1)
    for _ in range(4):
        hd.begin_time_step()
        hd.scalar_transport(30)  # converge the pseudo-time iterations (outlet value lags one)
        rhs = s_ref.copy()
        rhs[0] += c * 1.0
        s_ref = np.linalg.solve(A, rhs)
    s, _ = hd.get_scalar()
    assert np.abs(s[order] - s_ref).max() < 1e-12


def test_steady_advection_reaches_the_inlet_value(oracle_binding):
    hd, mesh, _ = open_channel(oracle_binding, 30)
    fixed = np.array([p.name == "inlet" for p in mesh.patches], np.int32)
    hd.scalar_enable(np.zeros(mesh.n_cells), fixed, np.where(fixed, 0.7, 0.0), recon=3)
    hd.scalar_transport(40)
    s, _ = hd.get_scalar()
    assert np.abs(s - 0.7).max() < 1e-8


def test_scalar_errors(oracle_binding):
    hd, mesh, _ = open_channel(oracle_binding, 10)
    with pytest.raises(abi.IcsError) as e:
        hd.scalar_transport(1)
    assert e.value.status == abi.ICS_ERR_STATE
    with pytest.raises(abi.IcsError):
        hd.scalar_enable(np.zeros(mesh.n_cells), recon=9)
