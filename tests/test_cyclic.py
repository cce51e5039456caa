"""Cyclic (coupled) patches: geometry and the oracle against a doubled domain (CPU).

A cyclic pair makes a periodic mesh; a state with the period of the short
domain must give the short domain's residual, local time step and Jacobian
action in the cells of a domain twice as long, where the coupled faces of the
short one are ordinary internal faces.  Checked for

* a translational cyclic (bump channel periodic across its span; any
  velocity field), every flux scheme, MUSCL/Venkatakrishnan and TVD vanLeer;
* a rotational cyclic (20-degree annular sector against the 40-degree one):
  the partner's gradients and velocity are rotated into the face's frame.
  The reference reconstructs U component by component, and a scalar
  component field's cyclic neighbour values are not rotated, so the state
  here is axial (the components are frame-independent) with theta-periodic
  scalar fields; the Jacobian action is checked on a vector whose momentum
  is periodic in cylindrical components.
* the viscous terms (Gauss gradients of U and e, laplacians with the
  non-orthogonal correction, div(tauMC), div(sigmaDotU . S), the LF viscous
  Jacobian) across both kinds of pair.
"""

import numpy as np
import pytest

from icsfoam_gb300 import abi, cases
from icsfoam_gb300 import mesh as M


def _open(b, mesh, settings, p, U, T):
    h = abi.CaseHandle(b, mesh, cases.make_config(b, settings))
    h.set_primitive(p, U, T)
    return h


def _bump(nz, width, periodic=True):
    g = cases.bump_points(8, 4, nz, width=width)
    inlet = M.Patch("inlet", M.PATCH_TOTAL_INLET, p0=1.0e5, T0=300.0)
    outlet = M.Patch("outlet", M.PATCH_PRESSURE_OUTLET, p=0.75e5)
    wall = M.Patch("walls", M.PATCH_SLIP, is_wall=True)
    a, b = M.cyclic_pair("front", "back", separation=(0.0, 0.0, -width))
    sides = {"xmin": inlet, "xmax": outlet, "ymin": wall, "ymax": wall, "zmin": a, "zmax": b}
    return M.hex_mesh(g, sides)


def _periodic_state(mesh, width):
    x, y, z = mesh.C.T
    # phases keep cell values off the limiters' ties (a neighbour equal to the
    # cell, extrapolations at round-off), where a 1e-17 change of the
    # geometry would switch a limiter branch
    s = np.sin(2 * np.pi * z / width + 0.4)
    c = np.cos(2 * np.pi * z / width + 1.1)
    p = 8.0e4 * (1 + 0.05 * np.sin(3 * x) * c + 0.03 * y * s + 0.01 * y)
    T = 280.0 * (1 + 0.04 * np.cos(2 * x + y) * s + 0.02 * x)
    U = np.stack([200 + 20 * np.sin(2 * x) * c + 9 * y, 15 * y * s + 5 * c + 3 * x,
                  25 * c * np.cos(x) + 11 * y + 4 * x], axis=1)
    return p, U, T


def _rows(small, big):
    """Index of each cell of ``small`` in ``big`` by generator index."""
    key = lambda m: m.cell_ijk[:, 0] + 1000 * (m.cell_ijk[:, 1] + 1000 * m.cell_ijk[:, 2])
    pos = {k: i for i, k in enumerate(key(big))}
    return np.array([pos[k] for k in key(small)])


def test_cyclic_geometry():
    m = _bump(3, 0.3)
    sel = m.b_partner >= 0
    assert sel.sum() == 2 * 8 * 4
    assert np.allclose(m.b_weights[sel], 0.5)
    # delta = distance between the cell centre and its partner across the span
    assert np.allclose(1.0 / m.b_delta_coeffs[sel], 0.1)
    with pytest.raises(ValueError):
        a, b = M.cyclic_pair("front", "back", separation=(0.0, 0.0, -0.25))
        g = cases.bump_points(8, 4, 3, width=0.3)
        M.hex_mesh(g, {"xmin": a, "xmax": b, "ymin": a, "ymax": b, "zmin": a, "zmax": b})


VISCOUS = dict(viscous=1, sutherland=1, As=1.458e-6, Ts=110.4, Pr=0.72)


@pytest.mark.parametrize("flux,recon,viscous", [("HLLC", 3, 0), ("AUSMPlusUp", 3, 0), ("ROE", 3, 0), ("HLLC", 1, 0),
                                                ("AUSMPlusUp", 0, 0), ("AUSMPlusUp", 3, 1), ("HLLC", 1, 1)])
def test_translational_cyclic_equals_doubled_span(oracle_binding, flux, recon, viscous):
    ma, mb = _bump(3, 0.3), _bump(6, 0.6)
    st = dict(cases.bump_channel(4, 2, 2, flux=flux).settings, recon_rho=recon, recon_U=recon, recon_T=recon,
              **(VISCOUS if viscous else {}))
    ha = _open(oracle_binding, ma, st, *_periodic_state(ma, 0.3))
    hb = _open(oracle_binding, mb, st, *_periodic_state(mb, 0.3))
    rows = _rows(ma, mb)
    ra, rb = ha.residual(), hb.residual()
    scale = np.abs(ra).max(axis=0)
    assert (np.abs(rb[rows] - ra) / scale).max() < 1e-10
    pa, pb = ha.get_pseudo_co()[1], hb.get_pseudo_co()[1]
    assert np.allclose(pb[rows], pa, rtol=1e-12)
    for h in (ha, hb):
        h.assemble_jacobian()
    x = _periodic_state(mb, 0.3)[1]
    xb = np.concatenate([x[:, :1] * 1e-3, x, x[:, 2:] * 7.0], axis=1)
    xa = xb[rows]
    ya, yb = ha.matrix_mul(xa), hb.matrix_mul(xb)
    assert (np.abs(yb[rows] - ya) / np.abs(ya).max(axis=0)).max() < 1e-10


def _sector_state(mesh):
    x, y, z = mesh.C.T
    r = np.hypot(x, y)
    th = np.arctan2(y, x)
    per = 2 * np.pi / np.radians(20.0)
    p = 9.0e4 * (1 + 0.05 * np.sin(per * th + 0.4) * np.cos(20 * z + 0.3) + 0.1 * (r - 0.55))
    T = 285.0 * (1 + 0.03 * np.cos(per * th + 1.0) * np.sin(15 * z + 0.2) + 0.2 * (r - 0.5) + 0.1 * z)
    U = np.zeros((mesh.n_cells, 3))
    U[:, 2] = 130.0 + 20.0 * np.sin(per * th + 0.7) * (r - 0.5) * 10 + 5 * np.cos(30 * z + 0.5) + 50 * (r - 0.5)
    return p, U, T, r, th


@pytest.mark.parametrize("flux,recon,viscous", [("HLLC", 3, 0), ("ROE", 1, 0), ("AUSMPlusUp", 3, 0),
                                                ("AUSMPlusUp", 3, 1)])
def test_rotational_cyclic_equals_doubled_sector(oracle_binding, flux, recon, viscous):
    wa = cases.annular_sector(4, 6, 5, sector_deg=20.0, ordering_mode="natural", flux=flux)
    wb = cases.annular_sector(4, 12, 5, sector_deg=40.0, theta0_deg=-10.0, ordering_mode="natural", flux=flux)
    st = dict(wa.settings, recon_rho=recon, recon_U=recon, recon_T=recon, **(VISCOUS if viscous else {}))
    pa, Ua, Ta, _, _ = _sector_state(wa.mesh)
    pb, Ub, Tb, rb_, thb = _sector_state(wb.mesh)
    ha = _open(oracle_binding, wa.mesh, st, pa, Ua, Ta)
    hb = _open(oracle_binding, wb.mesh, st, pb, Ub, Tb)
    rows = _rows(wa.mesh, wb.mesh)
    ra, rb = ha.residual(), hb.residual()
    scale = np.abs(ra).max(axis=0)
    scale[1:4] = scale[1:4].max()
    assert (np.abs(rb[rows] - ra) / scale).max() < 1e-10
    assert np.allclose(hb.get_pseudo_co()[1][rows], ha.get_pseudo_co()[1], rtol=1e-12)
    for h in (ha, hb):
        h.assemble_jacobian()
    # momentum periodic in cylindrical components
    per = 2 * np.pi / np.radians(20.0)
    er = np.stack([np.cos(thb), np.sin(thb), 0 * thb], axis=1)
    et = np.stack([-np.sin(thb), np.cos(thb), 0 * thb], axis=1)
    ar, at = np.sin(per * thb), np.cos(per * thb) * (rb_ - 0.5)
    mom = ar[:, None] * er + at[:, None] * et + np.sin(per * thb + 0.3)[:, None] * np.array([0, 0, 1.0])
    xb = np.concatenate([np.cos(per * thb)[:, None], mom, (1 + np.sin(per * thb))[:, None]], axis=1)
    ya, yb = ha.matrix_mul(xb[rows]), hb.matrix_mul(xb)
    sc = np.abs(ya).max(axis=0)
    sc[1:4] = sc[1:4].max()
    assert (np.abs(yb[rows] - ya) / sc).max() < 1e-10


def test_cyclic_rejects_a_viscous_scalar(oracle_binding):
    w = cases.annular_sector(3, 4, 4, ordering_mode="natural")
    h = _open(oracle_binding, w.mesh, dict(w.settings, **VISCOUS), w.p, w.U, w.T)
    with pytest.raises(abi.IcsError):
        h.scalar_enable(np.zeros(w.mesh.n_cells), D=1e-5)


@pytest.mark.parametrize("recon", [0, 3])
def test_scalar_across_translational_cyclic_equals_doubled_span(oracle_binding, recon):
    """Passive scalar: one transport step from a periodic s (block-Jacobi
    preconditioning, which both domains share) gives the short domain's s in
    the long one."""
    ma, mb = _bump(3, 0.3), _bump(6, 0.6)
    st = dict(cases.bump_channel(4, 2, 2).settings, preconditioner=2, max_iter=50, rel_tol=1e-12,
              tolerance=1e-30)
    out = []
    for m in (ma, mb):
        h = _open(oracle_binding, m, st, *_periodic_state(m, 0.3))
        x, y, z = m.C.T
        s0 = 0.5 + 0.3 * np.sin(2 * np.pi * z / 0.3 + 0.2) * np.cos(2 * x + 0.1) + 0.1 * y
        fixed = np.array([p.name == "inlet" for p in m.patches], np.int32)
        h.scalar_enable(s0, fixed, np.where(fixed == 1, 0.8, 0.0), recon=recon)
        h.scalar_transport(1)
        out.append(h.get_scalar()[0])
    rows = _rows(ma, mb)
    assert np.abs(out[1][rows] - out[0]).max() < 1e-10


def test_cyclic_case_files_round_trip(tmp_path, oracle_binding):
    """A rotational cyclic sector written as an OpenFOAM case (cyclic
    polyPatches with their transform) and read back: same coupled geometry,
    same residual."""
    from test_foam_case import write_dicts

    from icsfoam_gb300 import foam_case

    w = cases.annular_sector(3, 5, 4, ordering_mode="natural")
    foam_case.write_case(str(tmp_path), w.mesh, w.p, w.U, w.T)
    write_dicts(str(tmp_path))
    mesh, fields, settings, _ = foam_case.load_case(str(tmp_path))
    for k in ("b_partner", "b_weights", "b_nbr_d", "b_delta_coeffs", "b_nonorth_delta_coeffs"):
        assert np.allclose(getattr(mesh, k), getattr(w.mesh, k), rtol=1e-12, atol=1e-14), k
    rot = {p.name: np.asarray(p.rotation) for p in mesh.patches if p.rotation is not None}
    for p in w.mesh.patches:
        if p.kind == M.PATCH_CYCLIC:
            assert np.allclose(rot[p.name], p.rotation, atol=1e-14)
    h1 = _open(oracle_binding, w.mesh, w.settings, w.p, w.U, w.T)
    h2 = _open(oracle_binding, mesh, w.settings, fields["p"], fields["U"], fields["T"])
    r1, r2 = h1.residual(), h2.residual()
    assert np.abs(r1 - r2).max() <= 1e-11 * np.abs(r1).max()


LS89 = __import__("os").path.join("/", "root", "reference", "tutorials", "VKI-LS89")


@pytest.mark.skipif(not __import__("os").path.isdir(LS89), reason="reference tutorials not on this machine")
def test_reads_the_reference_cascade_with_translational_cyclics(oracle_binding):
    """The reference's VKI-LS89 turbine cascade (read in place, nothing
    copied): its pitch-wise periodicity is a translational cyclic pair; a
    laminar viscous pseudo iteration (the case's constant mu; its turbulence
    model is outside the path) runs through the oracle."""
    from icsfoam_gb300 import foam_case

    mesh, fields, settings, _ = foam_case.load_case(LS89)
    names = [p.name for p in mesh.patches]
    assert mesh.patches[names.index("Upper_periodicity")].kind == M.PATCH_CYCLIC
    sel = mesh.b_partner >= 0
    assert sel.sum() == 2 * 215
    assert np.all((mesh.b_weights[sel] > 0) & (mesh.b_weights[sel] < 1))
    assert settings.get("viscous", 0) == 1
    h = _open(oracle_binding, mesh, settings, fields["p"], fields["U"], fields["T"])
    h.begin_time_step()
    s = h.pseudo_iteration()
    assert np.isfinite(s.rho_l2_residual)
    assert np.all(np.isfinite(h.get_state()["W"]))
