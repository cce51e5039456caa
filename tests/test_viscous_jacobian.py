"""Viscous Jacobian without LaxFriedrichJacobian (CPU, the oracle).

``fvSchemes/viscousFluxScheme/LaxFriedrichJacobian false`` replaces the LF
stabilisation -- the scalar laplacian of 0.5 (mu + alphaEff)/rho on every
equation (viscousFluxScheme.C:234-247) -- by the laplacians of the face mu
and alphaEff acting on the conserved variables through -U/rho, 1/rho,
-E/rho + |U|^2/rho (viscousFluxScheme.C:249-267; the laplacian of
blockFvOperatorsTemplates.C:386-448 and :590-660), plus the diagonal
boundary terms of the physical patches, mu_b and alphaEff_b times the
patch fields' gradientInternalCoeffs (viscousFluxScheme.C:41-86, 120-215).

The difference of the two matrices' actions is restated here in numpy from
the mesh, the cell state and the boundary state, on the randomised viscous
box (fixedValue inlet, zeroGradient outlet and top, isothermal wall, slip
sides) and on the annular sector (total-pressure inlet, pressure outlet,
isothermal hub, slip shroud, rotational cyclic sides whose interface takes
the fields at the patch value and multiplies the partner's rotated
unknowns).
"""

import numpy as np
import pytest

from icsfoam_gb300 import abi, cases, schemes
from icsfoam_gb300 import mesh as M

from test_gpu_parity import perturb, relerr  # noqa: E402

VISCOUS = dict(viscous=1, sutherland=1, As=1.458e-6, Ts=110.4, Pr=0.72)


def workload(name):
    if name == "box":
        return perturb(cases.random_box(5))
    w = perturb(cases.annular_sector(4, 6, 5, ordering_mode="colour", flux="AUSMPlusUp"))
    names = [p.name for p in w.mesh.patches]
    w.mesh.patches[names.index("hub")].kind = M.PATCH_ISOTHERMAL_WALL
    w.mesh.patches[names.index("hub")].T = 290.0
    w.settings = dict(w.settings, **VISCOUS)
    return w


def open_case(b, w, **over):
    h = abi.CaseHandle(b, w.mesh, cases.make_config(b, w.settings, **over))
    h.set_primitive(w.p, w.U, w.T)
    return h


def _lap(fields, mg, ag, x):
    """The five laplacian blocks at the states ``fields`` = (-U/rho, 1/rho,
    -E/rho + |U|^2/rho) with coefficients mg (mu) and ag (alphaEff), times x."""
    mUr, ir, eR = fields
    y = np.zeros_like(x)
    y[:, 1:4] = mUr * (mg * x[:, 0])[:, None] + (ir * mg)[:, None] * x[:, 1:4]
    y[:, 4] = eR * ag * x[:, 0] + ag * np.sum(mUr * x[:, 1:4], axis=1) + ir * ag * x[:, 4]
    return y


def _fields(rho, U, T, Cv):
    u2 = np.sum(U * U, axis=1)
    E = Cv * T + 0.5 * u2
    return -U / rho[:, None], 1.0 / rho, -E / rho + u2 / rho


def expected_delta(w, st, bs, x):
    """(J without LF - J with LF) x from the mesh and the states."""
    m, s = w.mesh, w.settings
    R, Cp = s["R"], s["Cp"]
    Cv = Cp - R
    if s.get("sutherland"):
        mu = lambda T: s["As"] * np.sqrt(T) / (1.0 + s["Ts"] / T)  # noqa: E731
    else:
        mu = lambda T: np.full_like(T, s["mu"])  # noqa: E731
    alpha = lambda mu_: Cp / Cv * (mu_ / s["Pr"])  # noqa: E731
    rho, U, T = st["W"][:, 0], st["U"], st["T"]
    muc = mu(T)
    alc = alpha(muc)
    cell = _fields(rho, U, T, Cv)
    sel = lambda f, idx: tuple(a[idx] for a in f)  # noqa: E731
    y = np.zeros_like(x)
    # internal faces
    o, n, wf = m.owner, m.neighbour, m.weights
    lin = lambda a, b: wf * (a - b) + b  # noqa: E731
    muf, alf, rhof = lin(muc[o], muc[n]), lin(alc[o], alc[n]), lin(rho[o], rho[n])
    ms = np.linalg.norm(m.Sf, axis=1)
    mg, ag = muf * ms * m.delta_coeffs, alf * ms * m.delta_coeffs
    slf = 0.5 * ((muf + alf) / rhof) * ms * m.delta_coeffs
    lo, ln = _lap(sel(cell, o), mg, ag, x[o]), _lap(sel(cell, n), mg, ag, x[n])
    np.add.at(y, o, lo - ln - slf[:, None] * (x[o] - x[n]))
    np.add.at(y, n, ln - lo - slf[:, None] * (x[n] - x[o]))
    # boundary faces
    Bn = len(m.b_cell)
    kinds = np.array([m.patches[k].kind for k in m.b_patch])
    bo = m.b_cell
    bms = np.linalg.norm(m.b_Sf, axis=1)
    nf = m.b_Sf / bms[:, None]
    cyc = kinds == M.PATCH_CYCLIC
    if cyc.any():
        b = np.nonzero(cyc)[0]
        pc = m.b_partner[b]
        wb = m.b_weights[b]
        linb = lambda a, c: wb * (a - c) + c  # noqa: E731
        mufb, alfb, rhofb = linb(muc[bo[b]], muc[pc]), linb(alc[bo[b]], alc[pc]), linb(rho[bo[b]], rho[pc])
        dcb = m.b_delta_coeffs[b]
        mgb, agb = mufb * bms[b] * dcb, alfb * bms[b] * dcb
        slfb = 0.5 * ((mufb + alfb) / rhofb) * bms[b] * dcb
        Rm = np.array([np.reshape(m.patches[k].rotation, (3, 3)) for k in m.b_patch[b]])
        xr = x[pc].copy()
        xr[:, 1:4] = np.einsum("bij,bj->bi", Rm, x[pc, 1:4])
        rhoB = bs["p"][b] / (R * bs["T"][b])
        patch = _fields(rhoB, bs["U"][b], bs["T"][b], Cv)
        yb = _lap(sel(cell, bo[b]), mgb, agb, x[bo[b]]) - _lap(patch, mgb, agb, xr) - slfb[:, None] * (x[bo[b]] - xr)
        np.add.at(y, bo[b], yb)
    # physical patches: gradientInternalCoeffs of U and T
    dc = m.b_delta_coeffs
    uG = np.zeros((Bn, 3))
    tG = np.zeros(Bn)
    fixed = (kinds == M.PATCH_FIXED) | (kinds == M.PATCH_ISOTHERMAL_WALL)
    uG[fixed] = -dc[fixed, None]
    tG[fixed] = -dc[fixed]
    slip = kinds == M.PATCH_SLIP
    uG[slip] = -dc[slip, None] * np.abs(nf[slip])
    inl = kinds == M.PATCH_TOTAL_INLET
    tG[inl] = -dc[inl]
    infl = inl & (bs["phi"] < 0)
    uG[infl] = -dc[infl, None] * np.sqrt(np.abs(1.0 - nf[infl] ** 2))
    muB = mu(bs["T"])
    alB = alpha(muB)
    dM = -muB[:, None] * uG * bms[:, None]
    dE = -alB * Cv * tG * bms
    rI, UI, TI = rho[bo], U[bo], T[bo]
    u2 = np.sum(UI * UI, axis=1)
    EI = Cv * TI + 0.5 * u2
    xb = x[bo]
    yb = np.zeros((Bn, 5))
    yb[:, 1:4] = dM * (-UI / rI[:, None]) * xb[:, 0:1] + (dM / rI[:, None]) * xb[:, 1:4]
    yb[:, 4] = (dE * (-1.0 / (Cv * rI) * (EI - u2)) * xb[:, 0] + np.sum((dE / (Cv * rI))[:, None] * -UI * xb[:, 1:4], 1)
                + dE / (Cv * rI) * xb[:, 4])
    yb[cyc] = 0.0
    np.add.at(y, bo, yb)
    return y


@pytest.mark.parametrize("name", ["box", "sector"])
def test_non_lf_viscous_jacobian_restated(oracle_binding, name):
    w = workload(name)
    hl = open_case(oracle_binding, w, viscous_lf_jacobian=1)
    he = open_case(oracle_binding, w, viscous_lf_jacobian=0)
    for h in (hl, he):
        h.residual()
        h.assemble_jacobian()
    st, bs = he.get_state(), he.get_boundary_state()
    x = np.random.default_rng(2).standard_normal((w.mesh.n_cells, 5))
    full = he.matrix_mul(x)
    got = full - hl.matrix_mul(x)
    want = expected_delta(w, st, bs, x)
    # the difference is 1e-4 of the whole action: compare it to 9 digits, and
    # its error to the whole action's roundoff
    assert relerr(got, want) < 1e-9
    assert relerr(full + (got - want), full) < 1e-14
    # the two modes share everything but the viscous blocks
    assert np.abs(got).max() > 0


def test_non_lf_viscous_trajectory_converges(oracle_binding):
    """Pseudo iterations with the non-LF viscous Jacobian drive the residual down."""
    w = workload("box")
    h = open_case(oracle_binding, w, viscous_lf_jacobian=0)
    r0 = np.abs(h.residual()).max(axis=0)
    for _ in range(6):
        h.pseudo_iteration()
    r1 = np.abs(h.residual()).max(axis=0)
    assert np.all(np.isfinite(r1)) and r1[0] < r0[0]


def test_lax_friedrich_jacobian_switch_from_fvschemes(oracle_binding):
    base = {"convectiveFluxScheme": {"fluxScheme": "AUSMPlusUp"}}
    sol = {"flowSolver": {"solver": "GMRES", "GMRES": {"nDirections": 8, "tolerance": 1e-12, "relTol": 0.01}},
           "pseudoTime": {"pseudoTol": 1e-30, "pseudoTolRel": 1e-30}}
    assert schemes.config_from_dicts(oracle_binding, base, sol).viscous_lf_jacobian == 1
    for v, want in (("false", 0), ("off", 0), ("true", 1), (True, 1), ("no", 0)):
        d = dict(base, viscousFluxScheme={"LaxFriedrichJacobian": v})
        assert schemes.config_from_dicts(oracle_binding, d, sol).viscous_lf_jacobian == want


def test_viscous_jacobian_mode_validated(oracle_binding):
    w = cases.random_box(3)
    with pytest.raises(abi.IcsError):
        abi.CaseHandle(oracle_binding, w.mesh, cases.make_config(oracle_binding, w.settings, viscous_lf_jacobian=2))
