"""Harmonic Balance on the CUDA path against the oracle.

Same stacked case (3 instances, oscillating back pressure) in both
libraries: residual source with the -V D W term, Jacobian action with the
V D couplings, the per-instance norm factors / residuals of the solve, and a
run of pseudo iterations with the per-instance pseudotimeControl sequence.
Tolerances as in the other parity tests (FP64: 1e-12 for single kernels,
1e-10 for solves and trajectories; mixed precision looser).
"""

import numpy as np
import pytest

from icsfoam_gb300 import abi, cases

from test_gpu_parity import relerr  # noqa: E402

pytestmark = pytest.mark.gpu


def open_case(b, w, **over):
    h = abi.CaseHandle(b, w.mesh, cases.make_config(b, w.settings, **over))
    h.set_hb(*w.hb)
    h.set_primitive(w.p, w.U, w.T)
    return h


@pytest.fixture(scope="module")
def hbcase():
    return cases.hb_bump_channel(16, 6, 3, amplitude=0.1)


def test_hb_residual_and_matrix_action(gpu_binding, oracle_binding, hbcase):
    hg, ho = open_case(gpu_binding, hbcase), open_case(oracle_binding, hbcase)
    assert relerr(hg.residual(), ho.residual()) < 1e-12
    hg.assemble_jacobian()
    ho.assemble_jacobian()
    x = np.random.default_rng(1).standard_normal((hbcase.mesh.n_cells, 5))
    assert relerr(hg.matrix_mul(x), ho.matrix_mul(x)) < 1e-12
    assert relerr(hg.precondition(x), ho.precondition(x)) < 1e-12


def test_hb_solve_increment(gpu_binding, oracle_binding, hbcase):
    hg, ho = open_case(gpu_binding, hbcase), open_case(oracle_binding, hbcase)
    for h in (hg, ho):
        h.residual()
        h.assemble_jacobian()
    pg, dg, _ = hg.solve_increment()
    po, do, _ = ho.solve_increment()
    assert pg.n_iterations == po.n_iterations
    assert np.allclose(pg.init_res[:], po.init_res[:], rtol=1e-10, atol=0)
    assert relerr(dg, do) < 1e-10


@pytest.mark.parametrize("precision,tol", [(0, 1e-10), (1, 1e-4)])
def test_hb_pseudo_iterations_and_loop(gpu_binding, oracle_binding, precision, tol):
    """Lockstep pseudo iterations; the loop completes and restarts (steady).

    24x8x4 instances: on this mesh the oracle's own trajectory moves by
    ~1e-14 under a 1e-14 perturbation of the initial state.  (Meshes such
    as 16x6x3 are ill-conditioned: a cell at a local extremum whose face
    extrapolation is round-off decides between limiter 0 and 1, and a 1e-14
    perturbation moves the oracle's own state by 5e-4 in one iteration.)
    """
    w = cases.hb_bump_channel(24, 8, 4, amplitude=0.1)
    over = dict(n_pseudo_corr_min=2, pseudo_tol=0.3, pseudo_tol_rel=1e-30)
    hg = open_case(gpu_binding, w, precision=precision, **over)
    ho = open_case(oracle_binding, w, **over)
    seq = []
    for _ in range(12):
        mg, mo = hg.pseudo_loop(), ho.pseudo_loop()
        assert mg == mo
        seq.append(mg)
        hg.pseudo_iteration()
        ho.pseudo_iteration()
        assert relerr(hg.get_state()["W"], ho.get_state()["W"]) < tol
    assert not all(seq)


def test_hb_rejects_noalloc_entry(gpu_binding, hbcase):
    import torch

    h = open_case(gpu_binding, hbcase)
    h.residual()
    h.assemble_jacobian()
    x = torch.zeros((hbcase.mesh.n_cells, 5), dtype=torch.float64, device="cuda")
    r = torch.zeros_like(x)
    l1 = torch.zeros(5, dtype=torch.float64, device="cuda")
    assert h.linear_residual_noalloc(x.data_ptr(), r.data_ptr(), l1.data_ptr()) == abi.ICS_ERR_ARG


@pytest.mark.parametrize("precision,tol", [(0, 1e-10), (1, 5e-3)])
def test_hb_solve_with_fused_operator(gpu_binding, oracle_binding, precision, tol):
    """6,144 cells on the two-level colour schedule: the GMRES cycle applies
    M^-1 A in the fused three-pass form (with the instance couplings)."""
    w = cases.hb_bump_channel(32, 16, 4, amplitude=0.1)
    hg = open_case(gpu_binding, w, precision=precision)
    ho = open_case(oracle_binding, w)
    for h in (hg, ho):
        h.residual()
        h.assemble_jacobian()
    pg, dg, _ = hg.solve_increment()
    po, do, _ = ho.solve_increment()
    if precision == 0:
        assert pg.n_iterations == po.n_iterations
    assert relerr(dg, do) < tol


def test_hb_zone_and_cylindrical_source_parity(gpu_binding, oracle_binding):
    """HB zone (upstream half) and cylCoords on instances with rotated meshes
    (differing cylindrical frames): residual, Jacobian, matrix action,
    LU-SGS, solve and a short trajectory against the oracle; the reverse-mode
    product stays the transpose of the forward one through the zone and the
    cylindrical frames."""
    from test_hb import _zone_case

    w, zone = _zone_case()

    def opened(b):
        h = abi.CaseHandle(b, w.mesh, cases.make_config(b, w.settings))
        h.set_hb(*w.hb)
        h.set_primitive(w.p, w.U, w.T)
        h.set_hb_zone(zone, True, (0.0, 0.0, 1.0), (0.0, 0.0, 0.0))
        return h

    hg, ho = opened(gpu_binding), opened(oracle_binding)
    assert relerr(hg.residual(), ho.residual()) < 1e-12
    hg.assemble_jacobian()
    ho.assemble_jacobian()
    Dg, _, _ = hg.get_jacobian()
    Do, _, _ = ho.get_jacobian()
    assert relerr(Dg, Do) < 1e-12
    x = np.random.default_rng(1).standard_normal((w.mesh.n_cells, 5))
    assert relerr(hg.matrix_mul(x), ho.matrix_mul(x)) < 1e-12
    assert relerr(hg.precondition(x), ho.precondition(x)) < 1e-12
    for it in range(3):
        sg, so = hg.pseudo_iteration(), ho.pseudo_iteration()
        assert sg.perf.n_iterations == so.perf.n_iterations
        assert relerr(hg.get_state()["W"], ho.get_state()["W"]) < 1e-10, it
    rng = np.random.default_rng(3)
    W = hg.get_state()["W"]
    for s in range(2):
        v = rng.standard_normal(W.shape) * np.abs(W).max(axis=0)
        u = rng.standard_normal(W.shape)
        Jv = hg.jvp(v)
        lhs, rhs = float(np.sum(u * Jv)), float(np.sum(hg.vjp_recompute(u) * v))
        assert abs(lhs - rhs) <= 1e-12 * np.linalg.norm(u) * np.linalg.norm(Jv)
