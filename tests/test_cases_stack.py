"""Stacking independent cases into one mesh (mesh.stack, cases.stack_cases),
on the CPU with the oracle.

The stacked mesh is the disjoint union of the cases: the oracle's residual,
Jacobian action and LU-SGS on the stack equal, row for row, those of each
case alone (1e-14 of each equation's max-norm; the cells of a case see only
their own faces, in their own order).  This is the property the GPU's
stacked-case mode rests on.
"""

import numpy as np

from icsfoam_gb300 import abi, cases

from test_gpu_parity import perturb, relerr  # noqa: E402


def _cases():
    return [perturb(cases.bump_channel(6, 4, 2, ordering_mode="colour"), seed=1),
            perturb(cases.bump_channel(9, 5, 3, ordering_mode="colour"), seed=2),
            perturb(cases.bump_channel(7, 4, 2, ordering_mode="natural"), seed=3)]


def _open(b, w):
    h = abi.CaseHandle(b, w.mesh, cases.make_config(b, w.settings))
    h.set_primitive(w.p, w.U, w.T)
    return h


def test_stack_layout():
    ws = _cases()
    w, start = cases.stack_cases(ws)
    m = w.mesh
    assert list(start) == [0] + list(np.cumsum([x.mesh.n_cells for x in ws]))
    assert m.n_faces == sum(x.mesh.n_faces for x in ws)
    assert m.n_bfaces == sum(x.mesh.n_bfaces for x in ws)
    assert len(m.patches) == sum(len(x.mesh.patches) for x in ws)
    case_of = np.repeat(np.arange(len(ws)), np.diff(start))
    assert np.array_equal(case_of[m.owner], case_of[m.neighbour])
    assert np.all(m.owner < m.neighbour)
    assert np.array_equal(w.p, np.concatenate([x.p for x in ws]))


def test_stacked_residual_matvec_and_lusgs_are_the_cases(oracle_binding):
    ws = _cases()
    w, start = cases.stack_cases(ws)
    hs = _open(oracle_binding, w)
    r = hs.residual()
    hs.assemble_jacobian()
    x = np.random.default_rng(4).standard_normal((w.mesh.n_cells, 5))
    y = hs.matrix_mul(x)
    z = hs.precondition(x)
    for k, wk in enumerate(ws):
        sl = slice(start[k], start[k + 1])
        h = _open(oracle_binding, wk)
        rk = h.residual()
        h.assemble_jacobian()
        assert relerr(r[sl], rk) < 1e-14
        assert relerr(y[sl], h.matrix_mul(x[sl])) < 1e-14
        assert relerr(z[sl], h.precondition(x[sl])) < 1e-14


def test_stack_refuses_cyclic_and_mixed_dimensions():
    import pytest

    from icsfoam_gb300 import mesh as M

    tube = cases.shock_tube(20).mesh        # 1-D: y and z empty
    bump = cases.bump_channel(4, 2, 2).mesh  # 3-D
    with pytest.raises(ValueError):
        M.stack([tube, bump])
    sector = cases.annular_sector(2, 4, 4, sides="cyclic").mesh
    with pytest.raises(ValueError):
        M.stack([sector, sector])
    with pytest.raises(ValueError):
        M.stack([])
