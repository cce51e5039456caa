"""Moving reference frames: host set-up and the oracle's MRF terms (CPU).

* frame fields of the annular sector's rotor: the zone's face velocities
  close (sum of u_MRF |S| over every cell vanishes: Omega x r is
  divergence-free and the faces are planar), hub and shroud carry no normal
  frame velocity, the side planes carry omega r, the boundary assignment is
  Omega x Cf on the included faces and absent on a non-rotating patch;
* zone dictionaries (MRFProperties / MRFTranslatingProperties layout);
* the oracle's source -(omega x rho U) V and its skew Jacobian block are
  exactly the difference between a zone with omega and the same zone with
  omega = 0 (same face velocities), and the boundary assignment follows
  dbnsFoam's sequence (each time step; fixed-value patches keep it).
"""

import numpy as np
import pytest

from icsfoam_gb300 import abi, cases
from icsfoam_gb300 import mesh as M
from icsfoam_gb300 import mrf as MRF
from icsfoam_gb300 import foam_case


@pytest.fixture(scope="module")
def sector():
    return cases.annular_sector(6, 8, 9, ordering_mode="natural", sides="slip")


def test_frame_fields_closure_and_patches(sector):
    m = sector.mesh
    zone = sector.mrf[0][0]
    om, fv, bU, inc = MRF.frame_fields(m, *sector.mrf)
    F = m.n_faces
    ms = np.linalg.norm(m.Sf, axis=1)
    bms = np.linalg.norm(m.b_Sf, axis=1)
    div = np.zeros(m.n_cells)
    np.add.at(div, m.owner, fv[:F] * ms)
    np.add.at(div, m.neighbour, -fv[:F] * ms)
    np.add.at(div, m.b_cell, fv[F:] * bms)
    scale = np.abs(fv).max() * ms.max()
    assert np.abs(div).max() < 1e-12 * scale
    assert np.array_equal(np.nonzero(om[:, 2])[0], np.nonzero(zone.cells)[0])
    assert np.all(om[zone.cells, 2] == zone.omega)
    names = [p.name for p in m.patches]
    inzone = zone.cells[m.b_cell]
    for nm in ("hub", "shroud"):
        sel = (m.b_patch == names.index(nm)) & inzone
        assert sel.any() and np.abs(fv[F:][sel]).max() < 1e-12 * zone.omega
        assert np.all(inc[sel] == 1)
    sel = (m.b_patch == names.index("sides")) & inzone
    r = np.hypot(m.b_Cf[sel, 0], m.b_Cf[sel, 1])
    assert np.allclose(np.abs(fv[F:][sel]), zone.omega * r, rtol=1e-12)  # Omega x Cf is normal to the planes
    Om = np.array([0, 0, zone.omega])
    assert np.allclose(bU[inc == 1], np.cross(Om, m.b_Cf[inc == 1]))
    assert not inc[~inzone].any()
    # a non-rotating hub keeps its face velocity entries but loses the assignment
    z2 = MRF.RotatingZone(zone.cells, zone.origin, zone.axis, zone.omega, non_rotating_patches=("hub",))
    om2, fv2, bU2, inc2 = MRF.frame_fields(m, [z2])
    hub = m.b_patch == names.index("hub")
    assert not inc2[hub].any() and np.array_equal(inc2[~hub], inc[~hub])
    assert np.array_equal(fv2, fv)
    with pytest.raises(KeyError):
        MRF.frame_fields(m, [MRF.RotatingZone(zone.cells, zone.origin, zone.axis, 1.0, ("nope",))])


def test_translating_zone_adds_and_relative_velocity(sector):
    m = sector.mesh
    V = np.array([1.0, 2.0, 3.0])
    cells = np.arange(10)
    t = MRF.TranslatingZone(cells, tuple(V))
    om, fv, bU, inc = MRF.frame_fields(m, [], [t])
    assert not om.any()
    zc = np.zeros(m.n_cells, bool)
    zc[cells] = True
    internal = zc[m.owner] | zc[m.neighbour]
    n = m.Sf / np.linalg.norm(m.Sf, axis=1)[:, None]
    assert np.allclose(fv[:m.n_faces][internal], n[internal] @ V)
    assert not fv[:m.n_faces][~internal].any()
    assert np.allclose(bU[inc == 1], V)
    U = np.ones((m.n_cells, 3))
    Ur = MRF.relative_velocity(m, U, sector.mrf[0], [t])
    assert not sector.mrf[0][0].cells[cells].any()
    assert np.allclose(Ur[cells], 1.0 - V)
    outside = ~zc & ~sector.mrf[0][0].cells
    assert np.array_equal(Ur[outside], U[outside])


def test_zones_from_dictionaries():
    text = """
    rotor
    {
        cellZone rotor;
        active yes;
        nonRotatingPatches (hub);
        origin (0 0 0);
        axis (0 0 2);
        omega constant 104.72;
    }
    """
    d = foam_case.parse_dict(text)
    rot, tra = MRF.zones_from_dicts(d, {"slider": {"cellZone": "rotor", "frameVelocity": "(1 0 0)"}},
                                    {"rotor": np.array([0, 1, 2])})
    assert len(rot) == 1 and len(tra) == 1
    assert rot[0].omega == 104.72 and tuple(rot[0].non_rotating_patches) == ("hub",)
    assert np.allclose(rot[0].Omega(), [0, 0, 104.72])
    assert tra[0].frame_velocity == (1.0, 0.0, 0.0)
    with pytest.raises(KeyError):
        MRF.zones_from_dicts({"z": {"cellZone": "missing", "origin": "(0 0 0)", "axis": "(0 0 1)",
                                    "omega": "1"}}, None, {})
    with pytest.raises(ValueError):
        MRF.zones_from_dicts({"z": {"cellZone": "rotor", "origin": "(0 0 0)", "axis": "(0 0 1)",
                                    "omega": "table ((0 0) (1 1))"}}, None, {"rotor": np.array([0])})


def _open(b, w, fields):
    h = abi.CaseHandle(b, w.mesh, cases.make_config(b, w.settings))
    h.set_primitive(w.p, w.U, w.T)
    h.set_mrf(fields)
    return h


def test_oracle_source_and_skew_block_are_the_omega_terms(oracle_binding):
    w = cases.annular_sector(6, 8, 9, ordering_mode="natural", sides="slip")
    rng = np.random.default_rng(0)
    w.U = w.U + rng.uniform(-20, 20, w.U.shape)
    om, fv, bU, inc = MRF.frame_fields(w.mesh, *w.mrf)
    h1 = _open(oracle_binding, w, (om, fv, bU, inc))
    h0 = _open(oracle_binding, w, (np.zeros_like(om), fv, bU, inc))
    r1, r0 = h1.residual(), h0.residual()
    st = h1.get_state()
    rhoU = st["W"][:, 1:4]
    expect = -np.cross(om, rhoU) * w.mesh.V[:, None]
    scale = np.abs(r0).max()
    assert np.abs((r1 - r0)[:, 1:4] - expect).max() < 1e-11 * scale
    assert np.array_equal(r1[:, [0, 4]], r0[:, [0, 4]])
    for h in (h0, h1):
        h.assemble_jacobian()
    D1, L1, U1 = h1.get_jacobian()
    D0, L0, U0 = h0.get_jacobian()
    assert np.array_equal(L1, L0) and np.array_equal(U1, U0)
    V = w.mesh.V
    sk = np.zeros((w.mesh.n_cells, 5, 5))
    sk[:, 1, 2], sk[:, 1, 3] = -om[:, 2] * V, om[:, 1] * V
    sk[:, 2, 1], sk[:, 2, 3] = om[:, 2] * V, -om[:, 0] * V
    sk[:, 3, 1], sk[:, 3, 2] = -om[:, 1] * V, om[:, 0] * V
    assert np.abs((D1 - D0) - sk).max() < 1e-12 * np.abs(D0).max()


def test_oracle_boundary_assignment_sequence(oracle_binding):
    """Slip faces get the frame velocity at each time step and lose it at
    the next boundary update; an isothermal wall keeps it."""
    w = cases.annular_sector(6, 8, 9, ordering_mode="natural", sides="slip")
    names = [p.name for p in w.mesh.patches]
    w.mesh.patches[names.index("hub")].kind = M.PATCH_ISOTHERMAL_WALL
    w.mesh.patches[names.index("hub")].T = 280.0
    om, fv, bU, inc = MRF.frame_fields(w.mesh, *w.mrf)
    h = _open(oracle_binding, w, (om, fv, bU, inc))
    sides = (w.mesh.b_patch == names.index("sides")) & (inc == 1)
    hub = (w.mesh.b_patch == names.index("hub")) & (inc == 1)
    assert np.array_equal(h.get_boundary_state()["U"][sides], bU[sides])
    h.begin_time_step()
    h.pseudo_iteration()
    b = h.get_boundary_state()
    assert np.array_equal(b["U"][hub], bU[hub])
    n = w.mesh.b_Sf[sides] / np.linalg.norm(w.mesh.b_Sf[sides], axis=1)[:, None]
    assert np.abs(np.einsum("ij,ij->i", b["U"][sides], n)).max() < 1e-10  # slip value again
    h.begin_time_step()
    assert np.array_equal(h.get_boundary_state()["U"][sides], bU[sides])


def test_case_files_round_trip(tmp_path):
    """cellZones + MRFProperties + MRFTranslatingProperties written and read
    back give the same frame fields (natural order) and the same zones under
    a renumbering."""
    from test_foam_case import write_dicts

    w = cases.annular_sector(4, 6, 9, ordering_mode="natural", sides="slip")
    rot = w.mrf[0][0]
    rot.non_rotating_patches = ("hub",)
    tra = MRF.TranslatingZone(np.nonzero(w.mesh.C[:, 2] < 0.05)[0], (1.0, 0.0, 2.0), ("inlet",))
    foam_case.write_case(str(tmp_path), w.mesh, w.p, w.U, w.T)
    foam_case.write_mrf(str(tmp_path), w.mesh, [rot], [tra])
    write_dicts(str(tmp_path))
    mesh, fields, settings, dicts = foam_case.load_case(str(tmp_path))
    r2, t2 = dicts["mrf_zones"]
    assert len(r2) == 1 and len(t2) == 1 and tuple(r2[0].non_rotating_patches) == ("hub",)
    a = MRF.frame_fields(w.mesh, [rot], [tra])
    b = MRF.frame_fields(mesh, r2, t2)
    for x, y in zip(a, b):
        assert np.allclose(x, y, rtol=1e-13, atol=1e-12)
    mesh3, _, _, d3 = foam_case.load_case(str(tmp_path), ordering_mode="colour")
    om3 = MRF.frame_fields(mesh3, *d3["mrf_zones"])[0]
    # the same cells, found by their centres
    key = lambda C: np.lexsort(np.round(C, 9).T)
    assert np.array_equal(om3[key(mesh3.C)], a[0][key(w.mesh.C)])
    assert MRF.frame_fields(mesh3, *d3["mrf_zones"])[3].sum() == a[3].sum()
