"""Moving reference frames (MRF zones) on the CUDA path against the oracle.

An annular sector with a rotating cell zone (middle third, omega about the
axis) and a perturbed initial state: face fluxes and residual source with
the relative normal velocities, pressure work and -(omega x rho U) V;
Jacobian blocks with -div(w, u_MRF |S|), the skew source block and the
relative boundary flux; a solve; a run of pseudo iterations (each one a
steady time step, so the frame velocity is re-assigned on the rotating
patches every time, as dbnsFoam's outerLoop.H does); the translating-zone
and Harmonic Balance (re-assignment after every update) variants; the
passive scalar; and the tangent of the residual against finite differences
of the oracle's.  Tolerances as in the other parity tests.
"""

import numpy as np
import pytest

from icsfoam_gb300 import abi, cases
from icsfoam_gb300 import mesh as M
from icsfoam_gb300 import mrf as MRF

from test_gpu_parity import perturb, relerr  # noqa: E402
from test_gpu_diff import direction, fd_jvp  # noqa: E402

pytestmark = pytest.mark.gpu

FLUXES = ["AUSMPlusUp", "HLLC", "ROE"]


def sector(flux="HLLC", **kw):
    return perturb(cases.annular_sector(6, 8, 9, ordering_mode="colour", flux=flux, sides="slip", **kw))


def open_case(b, w, mode=0, fields=None, **over):
    h = abi.CaseHandle(b, w.mesh, cases.make_config(b, w.settings, **over))
    if w.hb:
        h.set_hb(*w.hb)
    h.set_primitive(w.p, w.U, w.T)
    h.set_mrf(fields if fields is not None else MRF.frame_fields(w.mesh, *w.mrf), mode)
    return h


@pytest.mark.parametrize("flux", FLUXES)
def test_mrf_flux_residual_and_jacobian(gpu_binding, oracle_binding, flux):
    w = sector(flux)
    hg, ho = open_case(gpu_binding, w), open_case(oracle_binding, w)
    for a, b in zip(hg.calc_flux(), ho.calc_flux()):
        assert relerr(a, b) < 1e-12
    so, sg = ho.residual(), hg.residual()
    assert relerr(sg, so) < 1e-12
    assert relerr(hg.get_pseudo_co()[1], ho.get_pseudo_co()[1]) < 1e-12
    for h in (ho, hg):
        h.assemble_jacobian()
    Do, Lo, Uo = ho.get_jacobian()
    Dg, Lg, Ug = hg.get_jacobian()
    assert relerr(Dg, Do) < 1e-12
    assert relerr(Lg, Lo) < 1e-12
    assert relerr(Ug, Uo) < 1e-12
    x = np.random.default_rng(1).standard_normal((w.mesh.n_cells, 5))
    assert relerr(hg.matrix_mul(x), ho.matrix_mul(x)) < 1e-12


def test_mrf_changes_the_residual_and_jacobian(gpu_binding):
    """The zone's terms are live: the GPU residual and diagonal blocks move
    when the zone is switched on, and come back when it is switched off."""
    w = sector()
    h = abi.CaseHandle(gpu_binding, w.mesh, cases.make_config(gpu_binding, w.settings))
    h.set_primitive(w.p, w.U, w.T)
    r0 = h.residual()
    h.set_mrf(MRF.frame_fields(w.mesh, *w.mrf))
    r1 = h.residual()
    assert relerr(r1, r0) > 1e-6
    h.set_mrf(None)
    h.set_primitive(w.p, w.U, w.T)
    assert relerr(h.residual(), r0) == 0.0


@pytest.mark.parametrize("flux,precision,tol", [("HLLC", 0, 1e-10), ("AUSMPlusUp", 0, 1e-10), ("HLLC", 1, 1e-4)])
def test_mrf_pseudo_iterations(gpu_binding, oracle_binding, flux, precision, tol):
    w = sector(flux)
    hg = open_case(gpu_binding, w, precision=precision)
    ho = open_case(oracle_binding, w)
    for it in range(5):
        for h in (hg, ho):
            h.begin_time_step()
        sg, so = hg.pseudo_iteration(), ho.pseudo_iteration()
        assert abs(sg.rho_l2_residual - so.rho_l2_residual) <= tol * abs(so.rho_l2_residual), it
        assert relerr(hg.get_state()["W"], ho.get_state()["W"]) < tol, it
        bg, bo = hg.get_boundary_state(), ho.get_boundary_state()
        assert relerr(bg["U"], bo["U"]) < tol


@pytest.mark.parametrize("flux,iterations", [("ROE", 0), ("HLLC", 3)])
def test_mrf_translating_zone_and_excluded_patch(gpu_binding, oracle_binding, flux, iterations):
    """A translating zone on top of the rotor, and the rotor's hub declared
    non-rotating (its faces keep the face velocity but not the boundary
    assignment).  The Roe variant is compared on one residual only: its
    third pseudo iteration moves the oracle's own state by 2e-3 under a
    1e-14 change of the initial pressure (a limiter switch at a round-off
    tie), so a trajectory there compares two branches, not two codes."""
    w = sector(flux)
    rot = w.mrf[0][0]
    rot.non_rotating_patches = ("hub",)
    zc = w.mesh.C[:, 2]
    tra = MRF.TranslatingZone(cells=zc < 0.05, frame_velocity=(3.0, -2.0, 5.0))
    fields = MRF.frame_fields(w.mesh, [rot], [tra])
    hg, ho = open_case(gpu_binding, w, fields=fields), open_case(oracle_binding, w, fields=fields)
    assert relerr(hg.residual(), ho.residual()) < 1e-12
    for it in range(iterations):
        for h in (hg, ho):
            h.begin_time_step()
            h.pseudo_iteration()
        assert relerr(hg.get_state()["W"], ho.get_state()["W"]) < 1e-10


def test_mrf_fixed_patch_keeps_frame_velocity(gpu_binding, oracle_binding):
    """Isothermal-wall shroud (fixedValue U): the frame velocity assigned by
    correctBoundaryVelocity survives the boundary update; the viscous terms
    see it."""
    w = sector("AUSMPlusUp")
    pats = w.mesh.patches
    i = [p.name for p in pats].index("shroud")
    pats[i].kind, pats[i].T = M.PATCH_ISOTHERMAL_WALL, 300.0
    w.settings = dict(w.settings, viscous=1, sutherland=1, As=1.458e-6, Ts=110.4, Pr=0.72)
    hg, ho = open_case(gpu_binding, w), open_case(oracle_binding, w)
    for it in range(3):
        for h in (hg, ho):
            h.begin_time_step()
            h.pseudo_iteration()
        assert relerr(hg.get_state()["W"], ho.get_state()["W"]) < 1e-10
    bs = hg.get_boundary_state()
    sel = w.mesh.b_patch == i
    _, _, bU, inc = MRF.frame_fields(w.mesh, *w.mrf)
    on = sel & (inc == 1)
    assert on.any()
    assert np.array_equal(bs["U"][on], bU[on])


def test_mrf_harmonic_balance_every_update(gpu_binding, oracle_binding):
    """HB instances of the sector: omega only (zero face velocity) and the
    boundary velocity re-assigned after every update."""
    from icsfoam_gb300 import hb as HB
    base = sector()
    n = 3
    omegas = HB.omega_list([2.0 * np.pi * 50.0], [1])
    t = HB.select_instants(omegas, n, None)
    D = HB.hb_operator(omegas, t)
    st = HB.stack_instances(base.mesh, n)
    rep = lambda a: np.concatenate([a] * n)
    zone = base.mrf[0][0]
    zone_st = MRF.RotatingZone(cells=rep(zone.cells), origin=zone.origin, axis=zone.axis, omega=zone.omega)
    w = cases.Workload("hb_sector", st, rep(base.p), rep(base.U), rep(base.T), dict(base.settings), hb=(n, D))
    fields = MRF.frame_fields(st, [zone_st], [], harmonic_balance=True)
    assert not fields[1].any()
    hg = open_case(gpu_binding, w, mode=MRF.MODE_EVERY_UPDATE, fields=fields)
    ho = open_case(oracle_binding, w, mode=MRF.MODE_EVERY_UPDATE, fields=fields)
    assert relerr(hg.residual(), ho.residual()) < 1e-12
    for it in range(3):
        hg.pseudo_iteration()
        ho.pseudo_iteration()
        assert relerr(hg.get_state()["W"], ho.get_state()["W"]) < 1e-10
        bo = ho.get_boundary_state()
        assert relerr(hg.get_boundary_state()["U"], bo["U"]) < 1e-10
        inc = fields[3] == 1
        assert np.array_equal(bo["U"][inc], fields[2][inc])


def test_mrf_passive_scalar(gpu_binding, oracle_binding):
    w = sector("HLLC")
    hg, ho = open_case(gpu_binding, w), open_case(oracle_binding, w)
    s0 = 0.5 + 0.4 * np.sin(40.0 * w.mesh.C[:, 2]) * np.cos(30.0 * w.mesh.C[:, 1])
    fixed = np.array([p.name == "inlet" for p in w.mesh.patches], np.int32)
    for h in (hg, ho):
        h.scalar_enable(s0, fixed, np.where(fixed == 1, 0.9, 0.0), D=0.0, recon=3)
        h.begin_time_step()
        h.pseudo_iteration()
    pg, po = hg.scalar_transport(3), ho.scalar_transport(3)
    assert pg.n_iterations == po.n_iterations
    sg, so = hg.get_scalar()[0], ho.get_scalar()[0]
    assert np.abs(sg - so).max() < 1e-10


def test_mrf_tangent_matches_oracle_finite_differences(gpu_binding, oracle_binding):
    w = sector("HLLC")
    hs = []
    for b in (gpu_binding, oracle_binding):
        h = open_case(b, w)
        hs.append(h)
    # untie the boundary values (the limiters' max/min ties have no derivative)
    bs = hs[0].get_boundary_state()
    rng = np.random.default_rng(5)
    B = len(bs["p"])
    p = bs["p"] * (1 + 0.01 * rng.uniform(-1, 1, B))
    T = bs["T"] * (1 + 0.01 * rng.uniform(-1, 1, B))
    U = bs["U"] + rng.uniform(-1, 1, (B, 3))
    for h in hs:
        h.set_boundary_state(p, U, T, bs["phi"])
    hg, ho = hs
    W = hg.get_state()["W"]
    for seed in range(3):
        v = direction(W, seed)
        assert relerr(hg.jvp(v), fd_jvp(ho, W, v)) < 1e-5, seed
