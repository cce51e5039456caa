"""Cyclic (coupled) patches on the CUDA path against the oracle.

The 20-degree annular sector with its rotational cyclic side pair (and the
bump channel made periodic across its span): face fluxes, residual source
and local time step with the coupled faces reconstructed from the partner
cell; Jacobian blocks with the coupled diagonal part and the interface
product (partner rotation folded into the stored blocks); pseudo-iteration
trajectories in FP64 and mixed precision; the doubled-sector known answer on
the GPU; the rotating zone and Harmonic Balance on the cyclic sector; the
residual's tangent against finite differences of the oracle and the exact
Jacobian built from it.  Tolerances as in the other parity tests.
"""

import numpy as np
import pytest

from icsfoam_gb300 import abi, cases
from icsfoam_gb300 import mrf as MRF

from test_cyclic import _bump, _periodic_state, _rows, _sector_state  # noqa: E402
from test_gpu_diff import direction, fd_jvp  # noqa: E402
from test_gpu_parity import perturb, relerr  # noqa: E402

pytestmark = pytest.mark.gpu


def sector(flux="HLLC", **kw):
    return perturb(cases.annular_sector(6, 8, 9, ordering_mode="colour", flux=flux, **kw))


def open_case(b, w, mrf=False, **over):
    h = abi.CaseHandle(b, w.mesh, cases.make_config(b, w.settings, **over))
    if w.hb:
        h.set_hb(*w.hb)
    h.set_primitive(w.p, w.U, w.T)
    if mrf:
        h.set_mrf(MRF.frame_fields(w.mesh, *w.mrf))
    return h


@pytest.mark.parametrize("flux,recon", [("HLLC", 3), ("AUSMPlusUp", 3), ("ROE", 3), ("HLLC", 1), ("AUSMPlusUp", 0)])
def test_cyclic_flux_residual_and_jacobian(gpu_binding, oracle_binding, flux, recon):
    w = sector(flux)
    w.settings = dict(w.settings, recon_rho=recon, recon_U=recon, recon_T=recon)
    hg, ho = open_case(gpu_binding, w), open_case(oracle_binding, w)
    bg, bo = hg.get_boundary_state(), ho.get_boundary_state()
    for k in ("p", "U", "T"):
        assert relerr(bg[k], bo[k]) < 1e-14
    for a, b in zip(hg.calc_flux(), ho.calc_flux()):
        assert relerr(a, b) < 1e-12
    assert relerr(hg.residual(), ho.residual()) < 1e-12
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
    assert relerr(hg.precondition(x), ho.precondition(x)) < 1e-12


@pytest.mark.parametrize("precision,tol", [(0, 1e-10), (1, 1e-4)])
def test_cyclic_pseudo_iterations(gpu_binding, oracle_binding, precision, tol):
    w = sector("HLLC")
    hg = open_case(gpu_binding, w, precision=precision)
    ho = open_case(oracle_binding, w)
    for it in range(5):
        sg, so = hg.pseudo_iteration(), ho.pseudo_iteration()
        assert sg.perf.n_iterations == so.perf.n_iterations or precision
        assert relerr(hg.get_state()["W"], ho.get_state()["W"]) < tol, it


def test_translational_cyclic_bump(gpu_binding, oracle_binding):
    m = _bump(3, 0.3)
    st = dict(cases.bump_channel(4, 2, 2).settings)
    p, U, T = _periodic_state(m, 0.3)
    w = cases.Workload("bump_periodic", m, p, U, T, st)
    hg, ho = open_case(gpu_binding, w), open_case(oracle_binding, w)
    assert relerr(hg.residual(), ho.residual()) < 1e-12
    for it in range(3):
        hg.pseudo_iteration()
        ho.pseudo_iteration()
        assert relerr(hg.get_state()["W"], ho.get_state()["W"]) < 1e-10


def test_doubled_sector_known_answer_on_gpu(gpu_binding):
    wa = cases.annular_sector(4, 6, 5, sector_deg=20.0, ordering_mode="natural")
    wb = cases.annular_sector(4, 12, 5, sector_deg=40.0, theta0_deg=-10.0, ordering_mode="natural")
    pa, Ua, Ta, _, _ = _sector_state(wa.mesh)
    pb, Ub, Tb, _, _ = _sector_state(wb.mesh)
    ha = abi.CaseHandle(gpu_binding, wa.mesh, cases.make_config(gpu_binding, wa.settings))
    hb = abi.CaseHandle(gpu_binding, wb.mesh, cases.make_config(gpu_binding, wb.settings))
    ha.set_primitive(pa, Ua, Ta)
    hb.set_primitive(pb, Ub, Tb)
    rows = _rows(wa.mesh, wb.mesh)
    ra, rb = ha.residual(), hb.residual()
    assert relerr(rb[rows], ra) < 1e-10


def test_cyclic_with_rotating_zone(gpu_binding, oracle_binding):
    w = sector("AUSMPlusUp")
    hg, ho = open_case(gpu_binding, w, mrf=True), open_case(oracle_binding, w, mrf=True)
    assert relerr(hg.residual(), ho.residual()) < 1e-12
    for it in range(3):
        for h in (hg, ho):
            h.begin_time_step()
            h.pseudo_iteration()
        assert relerr(hg.get_state()["W"], ho.get_state()["W"]) < 1e-10


def test_cyclic_harmonic_balance(gpu_binding, oracle_binding):
    from icsfoam_gb300 import hb as HB
    base = sector()
    n = 3
    omegas = HB.omega_list([2.0 * np.pi * 50.0], [1])
    D = HB.hb_operator(omegas, HB.select_instants(omegas, n, None))
    st = HB.stack_instances(base.mesh, n)
    rep = lambda a: np.concatenate([a] * n)
    w = cases.Workload("hb_sector", st, rep(base.p), rep(base.U), rep(base.T), dict(base.settings), hb=(n, D))
    hg, ho = open_case(gpu_binding, w), open_case(oracle_binding, w)
    assert relerr(hg.residual(), ho.residual()) < 1e-12
    for it in range(3):
        hg.pseudo_iteration()
        ho.pseudo_iteration()
        assert relerr(hg.get_state()["W"], ho.get_state()["W"]) < 1e-10


def test_cyclic_tangent_and_exact_jacobian(gpu_binding, oracle_binding):
    w = sector("HLLC")
    hs = [open_case(b, w) for b in (gpu_binding, oracle_binding)]
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
    nnz, ncol = hg.assemble_exact_jacobian()
    ptr, cols, blocks = hg.get_exact_jacobian()
    N = w.mesh.n_cells
    v = direction(W, 11)
    rows = np.repeat(np.arange(N), np.diff(ptr))
    jv = np.zeros((N, 5))
    np.add.at(jv, rows, np.einsum("jik,jk->ji", blocks, v[cols]))
    assert relerr(jv, hg.jvp(v)) < 1e-11
    u = rng.standard_normal((N, 5))
    jtu = hg.vjp(u)
    lhs, rhs = float(np.sum(u * hg.jvp(v))), float(np.sum(jtu * v))
    assert abs(lhs - rhs) <= 1e-11 * (np.abs(u * jv).sum() + np.abs(jtu * v).sum())


VISCOUS = dict(viscous=1, sutherland=1, As=1.458e-6, Ts=110.4, Pr=0.72)


@pytest.mark.parametrize("flux,precision,tol", [("AUSMPlusUp", 0, 1e-10), ("HLLC", 1, 1e-4)])
def test_cyclic_viscous(gpu_binding, oracle_binding, flux, precision, tol):
    """Viscous terms across the rotational cyclic pair: residual, Jacobian
    (with the coupled laplacian's interface) and a short trajectory."""
    w = sector(flux)
    names = [p.name for p in w.mesh.patches]
    w.mesh.patches[names.index("hub")].kind = 6  # isothermal no-slip hub
    w.mesh.patches[names.index("hub")].T = 290.0
    w.settings = dict(w.settings, **VISCOUS)
    hg = open_case(gpu_binding, w, precision=precision)
    ho = open_case(oracle_binding, w)
    if precision == 0:
        assert relerr(hg.residual(), ho.residual()) < 1e-12
        for h in (ho, hg):
            h.assemble_jacobian()
        Do, Lo, Uo = ho.get_jacobian()
        Dg, Lg, Ug = hg.get_jacobian()
        assert relerr(Dg, Do) < 1e-12
        x = np.random.default_rng(2).standard_normal((w.mesh.n_cells, 5))
        assert relerr(hg.matrix_mul(x), ho.matrix_mul(x)) < 1e-12
    for it in range(3):
        hg.pseudo_iteration()
        ho.pseudo_iteration()
        assert relerr(hg.get_state()["W"], ho.get_state()["W"]) < tol, it


def test_cyclic_viscous_tangent(gpu_binding, oracle_binding):
    w = sector("AUSMPlusUp")
    w.settings = dict(w.settings, **VISCOUS)
    hs = [open_case(b, w) for b in (gpu_binding, oracle_binding)]
    bs = hs[0].get_boundary_state()
    rng = np.random.default_rng(6)
    B = len(bs["p"])
    p = bs["p"] * (1 + 0.01 * rng.uniform(-1, 1, B))
    T = bs["T"] * (1 + 0.01 * rng.uniform(-1, 1, B))
    U = bs["U"] + rng.uniform(-1, 1, (B, 3))
    for h in hs:
        h.set_boundary_state(p, U, T, bs["phi"])
    W = hs[0].get_state()["W"]
    for seed in range(2):
        v = direction(W, seed)
        assert relerr(hs[0].jvp(v), fd_jvp(hs[1], W, v)) < 1e-5, seed


@pytest.mark.parametrize("recon,mrf", [(3, False), (1, True)])
def test_cyclic_passive_scalar(gpu_binding, oracle_binding, recon, mrf):
    w = sector("HLLC")
    hg, ho = open_case(gpu_binding, w, mrf=mrf), open_case(oracle_binding, w, mrf=mrf)
    x, y, z = w.mesh.C.T
    s0 = 0.5 + 0.4 * np.sin(40.0 * z + 0.3) * np.cos(30.0 * y + 0.1) + 0.2 * x
    fixed = np.array([p.name == "inlet" for p in w.mesh.patches], np.int32)
    for h in (hg, ho):
        h.scalar_enable(s0, fixed, np.where(fixed == 1, 0.9, 0.0), D=0.0, recon=recon)
        h.begin_time_step()
        h.pseudo_iteration()
    pg, po = hg.scalar_transport(3), ho.scalar_transport(3)
    assert pg.n_iterations == po.n_iterations
    assert np.abs(hg.get_scalar()[0] - ho.get_scalar()[0]).max() < 1e-10
