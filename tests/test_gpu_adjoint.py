"""Reverse-mode derivative of the residual (ics_vjp_recompute) on the GPU.

The reverse chain recomputes the fields, Gauss gradients and cellLimited
limiters in its backward pass and stores no Jacobian.  It must be the exact
transpose of the forward-mode product ics_jvp (<u, J v> = <J^T u, v> to
round-off, 1e-12 of |u| |J v|) and equal the product with the assembled exact
Jacobian (ics_vjp) to 1e-10 of each equation's max-norm, on every flux
scheme, both MUSCL limiters with and without the cellLimited coefficient,
both TVD limitedSchemes, first-order reconstruction, the unsteady (backward ddt) residual, Harmonic
Balance and an MRF zone.  Configurations it does not cover are refused.
"""

import numpy as np
import pytest

from icsfoam_gb300 import abi, cases
from icsfoam_gb300 import mrf as MRF

from test_gpu_diff import _over, direction, open_case  # noqa: E402
from test_gpu_parity import perturb, relerr  # noqa: E402

pytestmark = pytest.mark.gpu

REV = {
    "bump_hllc_muscl": lambda: cases.bump_channel(12, 6, 3, ordering_mode="colour", flux="HLLC"),
    "bump_hllc_muscl_k05": lambda: _over(cases.bump_channel(12, 6, 3, ordering_mode="colour", flux="HLLC"),
                                         limiter_coeff=0.5),
    "bump_ausm_muscl_minmod": lambda: _over(cases.bump_channel(10, 5, 3, ordering_mode="colour", flux="AUSMPlusUp"),
                                            recon_rho=4, recon_U=4, recon_T=4),
    "bump_roe_muscl": lambda: cases.bump_channel(10, 5, 3, ordering_mode="natural", flux="ROE"),
    "bump_roe_first_order": lambda: cases.bump_channel(10, 5, 3, ordering_mode="natural", flux="ROE",
                                                       second_order=False),
    "bump_roe_vanleer": lambda: _over(cases.bump_channel(10, 5, 3, ordering_mode="natural", flux="ROE"),
                                      recon_rho=1, recon_U=1, recon_T=1),
    "bump_hllc_minmod_tvd": lambda: _over(cases.bump_channel(12, 6, 3, ordering_mode="colour", flux="HLLC"),
                                          recon_rho=2, recon_U=2, recon_T=2),
    "tube_ausm_backward": lambda: cases.shock_tube(60),
    "hb_bump_hllc": lambda: cases.hb_bump_channel(8, 4, 2, amplitude=0.1),
    "mrf_sector_hllc": lambda: cases.annular_sector(4, 6, 6, ordering_mode="colour", flux="HLLC", sides="slip"),
}


def _open(b, name):
    w = perturb(REV[name]())
    h = open_case(b, w)
    if w.mrf:
        h.set_mrf(MRF.frame_fields(w.mesh, *w.mrf), 0)
    if w.settings.get("ddt_scheme", 0):
        for _ in range(2):  # the second step switches backward ddt to its BDF2 coefficients
            h.begin_time_step()
    return w, h


@pytest.mark.parametrize("name", list(REV))
def test_vjp_recompute_is_the_transpose_of_the_jvp(gpu_binding, name):
    w, h = _open(gpu_binding, name)
    W = h.get_state()["W"]
    rng = np.random.default_rng(3)
    for s in range(3):
        v = direction(W, 10 + s)
        u = rng.standard_normal(W.shape)
        Jv = h.jvp(v)
        JTu = h.vjp_recompute(u)
        lhs, rhs = float(np.sum(u * Jv)), float(np.sum(JTu * v))
        scale = np.linalg.norm(u) * np.linalg.norm(Jv)
        assert abs(lhs - rhs) <= 1e-12 * scale, (s, lhs, rhs)


@pytest.mark.parametrize("name", list(REV))
def test_vjp_recompute_equals_the_exact_jacobian_transpose(gpu_binding, name):
    w, h = _open(gpu_binding, name)
    u = np.random.default_rng(4).standard_normal((w.mesh.n_cells, 5))
    assert relerr(h.vjp_recompute(u), h.vjp(u)) < 1e-10


def test_vjp_recompute_refuses_what_it_does_not_cover(gpu_binding):
    w = perturb(cases.random_box(5))  # viscous
    h = open_case(gpu_binding, w)
    with pytest.raises(abi.IcsError):
        h.vjp_recompute(np.ones((w.mesh.n_cells, 5)))


def _swept(b, n=(24, 12, 8), iterations=3, precision=0, **over):
    """The swept bump after some pseudo iterations, with its approximate
    Jacobian assembled at that state (the preconditioner)."""
    w = cases.swept_bump(*n)
    h = abi.CaseHandle(b, w.mesh, cases.make_config(b, w.settings, precision=precision, **over))
    h.set_primitive(w.p, w.U, w.T)
    for _ in range(iterations):
        h.pseudo_loop()
        h.pseudo_iteration()
    h.residual()
    h.assemble_jacobian()
    bump = [p.name for p in w.mesh.patches].index("bump")
    return w, h, bump


def test_pressure_force_gradient_matches_finite_differences(gpu_binding):
    w, h, bump = _swept(gpu_binding)
    J0, g = h.pressure_force(bump, (1.0, 0.0, 0.0))
    W = h.get_state()["W"]
    for s in range(3):
        v = direction(W, 20 + s)
        eps = 1e-7
        h.set_conservative(W + eps * v)
        jp, _ = h.pressure_force(bump, (1.0, 0.0, 0.0), gradient=False)
        h.set_conservative(W - eps * v)
        jm, _ = h.pressure_force(bump, (1.0, 0.0, 0.0), gradient=False)
        h.set_conservative(W)
        fd = (jp - jm) / (2 * eps)
        assert abs(fd - float(np.sum(g * v))) <= 1e-6 * abs(fd), s


def _residuals(h, psi, x, g, b, pseudo_time):
    """True residuals of A^T psi = g and A x = b, A = s V/dtau - d(R V)/dW."""
    V = h.mesh.V[:, None]
    rp = h.get_pseudo_co()[1][:, None] if pseudo_time else 0.0
    r_a = (rp * V * psi - h.vjp_recompute(psi)) - g
    r_t = (rp * V * x - h.jvp(x)) - b
    return r_a, r_t


FIRST_ORDER = {"recon_rho": 0, "recon_U": 0, "recon_T": 0}


@pytest.mark.parametrize("pseudo_time,precision,iterations,over", [(1, 0, 3, {}), (1, 1, 3, {}),
                                                                   (1, 0, 3, FIRST_ORDER)])
def test_adjoint_and_tangent_solves_are_dual(gpu_binding, pseudo_time, precision, iterations, over):
    """A^T psi = g (reverse-mode operator) and A x = b (forward-mode operator,
    matrix-free Newton-Krylov), right-preconditioned by the approximate
    Jacobian's LU-SGS (transposed for the adjoint), solved to 1e-8 with an
    FP64 or FP32 Krylov basis, with the pseudo-time diagonal (the operator of
    the implicit pseudo-time step) early in the run.  The
    true residuals meet the tolerance and <g, x> = <psi, b> holds to the
    bound the two residuals allow, which needs the two operators to be each
    other's transpose."""
    w, h, bump = _swept(gpu_binding, iterations=iterations, **over)
    _, g = h.pressure_force(bump, (1.0, 0.0, 0.0))
    W = h.get_state()["W"]
    b = direction(W, 30) * 1e-3
    opts = dict(n_directions=40, max_cycles=60, rel_tol=1e-8, precision=precision, pseudo_time=pseudo_time)
    psi, ra = h.adjoint_solve(g, **opts)
    x, rt = h.tangent_solve(b, **opts)
    assert ra.converged and rt.converged, (ra.rel_residual, ra.iterations, rt.rel_residual, rt.iterations)
    r_a, r_t = _residuals(h, psi, x, g, b, pseudo_time)
    assert np.linalg.norm(r_a) <= 2e-8 * np.linalg.norm(g)
    assert np.linalg.norm(r_t) <= 2e-8 * np.linalg.norm(b)
    lhs, rhs = float(np.sum(g * x)), float(np.sum(psi * b))
    bound = np.linalg.norm(psi) * np.linalg.norm(r_t) + np.linalg.norm(r_a) * np.linalg.norm(x)
    assert abs(lhs - rhs) <= 2 * bound + 1e-12 * abs(lhs), (lhs, rhs, bound)


def test_steady_linearisation_at_convergence_is_singular(gpu_binding):
    """Why the Krylov solves offer the pseudo-time operator: at a state the
    pseudo-time iteration has converged (bump channel 12x4x2, first order, a
    1e-9 drop of the rho residual) the steady linearisation -d(R V)/dW with
    the boundary values held fixed (the JVP's operator), each variable scaled
    by its largest magnitude, is numerically singular (smallest singular value
    below 1e-10 of the largest) and has eigenvalues left of the imaginary
    axis, so a Krylov solve of it from a generic right-hand side stalls."""
    w = _over(cases.bump_channel(12, 4, 2, ordering_mode="colour"), recon_rho=0, recon_U=0, recon_T=0)
    h = abi.CaseHandle(gpu_binding, w.mesh, cases.make_config(gpu_binding, w.settings))
    h.set_primitive(w.p, w.U, w.T)
    r0 = None
    for _ in range(2000):
        h.pseudo_loop()
        s = h.pseudo_iteration()
        r0 = r0 or s.rho_l2_residual
        if s.rho_l2_residual < 1e-9 * r0:
            break
    assert s.rho_l2_residual < 1e-9 * r0
    W = h.get_state()["W"]
    n = W.size
    A = np.zeros((n, n))
    for j in range(n):
        e = np.zeros(n)
        e[j] = 1.0
        A[:, j] = -h.jvp(e.reshape(W.shape)).ravel()
    S = np.tile(np.abs(W).max(axis=0), W.shape[0])
    As = A * S[None, :] / S[:, None]
    sv = np.linalg.svd(As, compute_uv=False)
    assert sv[-1] < 1e-10 * sv[0], (sv[-1], sv[0])
    assert np.sum(np.linalg.eigvals(As).real < 0) >= 1
