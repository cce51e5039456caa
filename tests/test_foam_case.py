"""OpenFOAM case I/O: dictionary parser, polyMesh/field round trips, and (when
the reference's tutorials are present on this machine) reading a real case."""

import os

import numpy as np
import pytest

from icsfoam_gb300 import abi, cases, foam_case
from icsfoam_gb300 import mesh as M

DICTS = {
    "fvSchemes": """
convectiveFluxScheme { fluxScheme HLLC; }
ddtSchemes { default dualTime rPseudoDeltaT steadyState; }
gradSchemes { default Gauss linear; limited cellLimited<Venkatakrishnan> Gauss linear 1; }
interpolationSchemes
{
    default linear;
    reconstruct(rho) linearUpwind limited;
    reconstruct(U)   linearUpwind limited;
    reconstruct(T)   linearUpwind limited;
}
""",
    "fvSolution": """
flowSolver
{
    solver GMRES;
    GMRES { preconditioner LUSGS; nDirections 8; maxIter 5; tolerance 1e-12; relTol 1e-2; }
}
pseudoTime { nPseudoCorr 20; pseudoTol 1e-30; pseudoTolRel 1e-30; pseudoCoNum 1; pseudoCoNumMax 50; }
""",
    "thermophysicalProperties": """
thermoType { transport const; }
mixture
{
    specie { molWeight 28.9; }    // air
    thermodynamics { Cp 1004.5; Hf 0; }
    transport { mu 0; Pr 0.72; }
}
""",
}


def write_dicts(path):
    for name, text in DICTS.items():
        sub = "constant" if name.startswith("thermo") else "system"
        os.makedirs(os.path.join(path, sub), exist_ok=True)
        with open(os.path.join(path, sub, name), "w") as f:
            f.write("FoamFile { version 2.0; format ascii; class dictionary; object %s; }\n" % name)
            f.write(text)


def test_parse_dict_entries_and_blocks():
    d = foam_case.parse_dict("""
    /* block comment */ a 1; // line comment
    b { c "quoted"; d (1 2 3); e { f g h; } }
    ref $a;
    """)
    assert d["a"] == "1"
    assert d["b"]["c"] == '"quoted"'
    assert d["b"]["d"] == "( 1 2 3 )"
    assert d["b"]["e"]["f"] == "g h"
    assert d["ref"] == "1"


def _compare_meshes(a, b):
    assert a.n_cells == b.n_cells and a.n_faces == b.n_faces and a.n_bfaces == b.n_bfaces
    assert np.array_equal(a.owner, b.owner) and np.array_equal(a.neighbour, b.neighbour)
    for k in ("Sf", "Cf", "C", "V", "weights", "delta_coeffs", "nonorth_delta_coeffs", "b_Sf", "b_Cf"):
        assert np.allclose(getattr(a, k), getattr(b, k), rtol=1e-13, atol=1e-15), k
    assert tuple(a.solution_d) == tuple(b.solution_d)
    assert [p.kind for p in a.patches] == [p.kind for p in b.patches]


@pytest.mark.parametrize("make", [lambda: cases.bump_channel(6, 4, 3, ordering_mode="colour"),
                                  lambda: cases.shock_tube(20)])
def test_write_then_read_case(tmp_path, oracle_binding, make):
    w = make()
    foam_case.write_case(str(tmp_path), w.mesh, w.p, w.U, w.T)
    write_dicts(str(tmp_path))
    mesh, fields, settings, dicts = foam_case.load_case(str(tmp_path))
    _compare_meshes(w.mesh, mesh)
    for a, b in zip(w.mesh.patches, mesh.patches):
        assert (a.kind, a.is_wall, a.p, a.T, tuple(a.U), a.p0, a.T0) == (b.kind, b.is_wall, b.p, b.T, tuple(b.U),
                                                                           b.p0, b.T0)
    assert np.array_equal(fields["p"], w.p) and np.array_equal(fields["U"], w.U)
    assert settings["flux_scheme"] == 1 and settings["recon_U"] == 3 and settings["n_directions"] == 8
    assert abs(settings["R"] - 287.7) < 0.1 and settings["Cp"] == 1004.5
    # the same residual through the oracle on both meshes
    base = dict(w.settings)
    h1 = abi.CaseHandle(oracle_binding, w.mesh, cases.make_config(oracle_binding, base))
    h2 = abi.CaseHandle(oracle_binding, mesh, cases.make_config(oracle_binding, base))
    h1.set_primitive(w.p, w.U, w.T)
    h2.set_primitive(fields["p"], fields["U"], fields["T"])
    r1, r2 = h1.residual(), h2.residual()
    assert np.allclose(r1, r2, rtol=1e-12, atol=1e-12 * np.abs(r1).max())


def test_mixed_polygon_geometry():
    pts = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [0.5, 1.5, 0]], float)
    quads = np.array([[0, 1, 2, 3]])
    poly = np.empty(2, dtype=object)
    poly[0] = np.array([0, 1, 2, 3])
    poly[1] = np.array([3, 2, 4])  # triangle
    c1, s1 = M.face_centres_and_areas(pts, quads)
    c2, s2 = M.face_centres_and_areas(pts, poly)
    assert np.allclose(c2[0], c1[0]) and np.allclose(s2[0], s1[0])
    assert np.allclose(s2[1], [0, 0, 0.25]) and np.allclose(c2[1], [0.5, 7.0 / 6.0, 0])


def test_unsupported_boundary_conditions_raise():
    with pytest.raises(ValueError):
        foam_case.patch_from_bcs("x", "patch", {"type": "fixedValue", "value": "uniform 1"},
                                 {"type": "slip"}, {"type": "fixedValue", "value": "uniform 1"})
    with pytest.raises(ValueError):
        foam_case.patch_from_bcs("c", "cyclic", {"type": "cyclic"}, {"type": "cyclic"}, {"type": "cyclic"})


TUTORIAL = os.path.join(os.sep, "root", "reference", "tutorials", "forwardStep")


@pytest.mark.skipif(not os.path.isdir(TUTORIAL), reason="reference tutorials not on this machine")
def test_reads_a_reference_tutorial_case(oracle_binding):
    """The reference's forwardStep case (read in place, nothing copied) runs through the oracle."""
    mesh, fields, settings, dicts = foam_case.load_case(TUTORIAL)
    assert mesh.n_cells > 0 and tuple(mesh.solution_d)[2] == -1
    assert np.all(mesh.V > 0)
    kinds = {p.name: p.kind for p in mesh.patches}
    assert kinds["inlet"] == M.PATCH_FIXED and kinds["obstacle"] == M.PATCH_SLIP
    h = abi.CaseHandle(oracle_binding, mesh, cases.make_config(oracle_binding, settings))
    h.set_primitive(fields["p"], fields["U"], fields["T"])
    h.begin_time_step()
    s = h.pseudo_iteration()
    assert np.isfinite(s.rho_l2_residual)
    assert np.all(np.isfinite(h.get_state()["W"]))


@pytest.mark.gpu
def test_case_read_from_disk_runs_on_the_gpu(tmp_path, gpu_binding, oracle_binding):
    """A case written to disk and read back: GPU and oracle agree on it."""
    w = cases.bump_channel(24, 8, 4, ordering_mode="natural")
    foam_case.write_case(str(tmp_path), w.mesh, w.p, w.U, w.T)
    write_dicts(str(tmp_path))
    mesh, fields, settings, _ = foam_case.load_case(str(tmp_path), ordering_mode="colour")
    hs = []
    for b in (gpu_binding, oracle_binding):
        h = abi.CaseHandle(b, mesh, cases.make_config(b, settings))
        h.set_primitive(fields["p"], fields["U"], fields["T"])
        hs.append(h)
    for _ in range(3):
        for h in hs:
            h.pseudo_iteration()
    g, o = hs[0].get_state()["W"], hs[1].get_state()["W"]
    scale = np.abs(o).max(axis=0)
    scale[1:4] = scale[1:4].max()
    assert (np.abs(g - o) / scale).max() < 1e-9
