"""GPU path vs the CPU oracle on identical meshes and states (FP64 and mixed).

Tolerances (relative to the max-norm of the oracle quantity, per component):
  FP64 flux / residual / Jacobian / SpMV / LU-SGS:  1e-12
  FP64 GMRES increment and updated state:           1e-10
  mixed precision (FP32 blocks, preconditioner, Krylov basis):
      Jacobian blocks 1e-6, increment 5e-3 of max, updated state 1e-6
The FP64 bound allows for the different summation order of reductions and
the fused multiply-adds of the GPU; the algorithm is otherwise identical.
"""

import numpy as np
import pytest

from icsfoam_gb300 import cases, gpu

pytestmark = pytest.mark.gpu

WORKLOADS = {
    "tube_ausm_natural": lambda: cases.shock_tube(200),
    "bump_hllc_muscl_colour": lambda: cases.bump_channel(24, 8, 4, ordering_mode="colour", flux="HLLC"),
    "bump_ausm_muscl_colour": lambda: cases.bump_channel(24, 8, 4, ordering_mode="colour", flux="AUSMPlusUp"),
    "bump_roe_muscl_natural": lambda: cases.bump_channel(16, 6, 3, ordering_mode="natural", flux="ROE"),
    "box_ausm_rcm": lambda: cases.random_box(6),
    # large enough for per-level LU-SGS launches (fused last forward / first reverse level)
    "bump_hllc_muscl_colour_levels": lambda: cases.bump_channel(32, 16, 10, ordering_mode="colour", flux="HLLC"),
}

EXTRA = {
    "bump_hllc_vanleer_natural": dict(recon_rho=1, recon_U=1, recon_T=1),
    # cellLimited<Venkatakrishnan> Gauss linear 0.5
    "bump_hllc_muscl_k05_natural": dict(limiter_coeff=0.5),
}


def relerr(a, b):
    """Max error relative to the max-norm of each equation of the reference.

    Cell 5-vectors (n, 5): scales per equation with the three momentum
    components sharing one scale.  Blocks (n, 5, 5): scales per block row
    (equation), momentum rows shared.  Other arrays: one scale per column.
    """
    a = np.asarray(a, float)
    b = np.asarray(b, float)
    if b.ndim == 3 and b.shape[1:] == (5, 5):
        rows = np.abs(b).max(axis=(0, 2))
        rows[1:4] = rows[1:4].max()
        scale = np.broadcast_to(rows[None, :, None], b.shape)
    elif b.ndim == 2 and b.shape[1] == 5:
        cols = np.abs(b).max(axis=0)
        cols[1:4] = cols[1:4].max()
        scale = np.broadcast_to(cols[None, :], b.shape)
    else:
        b2 = b.reshape(len(b), -1)
        scale = np.broadcast_to(np.abs(b2).max(axis=0, keepdims=True), b2.shape).reshape(b.shape)
    scale = np.where(scale == 0, 1.0, scale)
    return float((np.abs(a - b) / scale).max())


def open_pair(oracle_binding, gpu_binding, w, **over):
    ho = cases_open(oracle_binding, w, **over)
    hg = cases_open(gpu_binding, w, **over)
    return ho, hg


def cases_open(binding, w, **over):
    from icsfoam_gb300 import abi

    cfg = cases.make_config(binding, w.settings, **over)
    h = abi.CaseHandle(binding, w.mesh, cfg)
    h.set_primitive(w.p, w.U, w.T)
    return h


def perturb(w, seed=3, amp=0.02):
    rng = np.random.default_rng(seed)
    N = w.mesh.n_cells
    w.p = w.p * (1 + amp * rng.uniform(-1, 1, N))
    w.T = w.T * (1 + amp * rng.uniform(-1, 1, N))
    w.U = w.U + amp * 100.0 * rng.uniform(-1, 1, (N, 3)) * (np.array(w.mesh.solution_d) > 0)
    return w


CASES = list(WORKLOADS) + list(EXTRA)


def make(name):
    if name in WORKLOADS:
        return perturb(WORKLOADS[name]()), {}
    return perturb(cases.bump_channel(16, 6, 3, ordering_mode="natural", flux="HLLC")), EXTRA[name]


@pytest.mark.parametrize("name", CASES)
def test_flux_and_residual(oracle_binding, gpu_binding, name):
    w, over = make(name)
    ho, hg = open_pair(oracle_binding, gpu_binding, w, **over)
    if w.settings.get("ddt_scheme", 0):
        ho.begin_time_step()
        hg.begin_time_step()
    fo, fg = ho.calc_flux(), hg.calc_flux()
    for a, b in zip(fg, fo):
        assert relerr(a, b) < 1e-12
    so, sg = ho.residual(), hg.residual()
    assert relerr(sg, so) < 1e-12
    co, ro = ho.get_pseudo_co()
    cg, rg = hg.get_pseudo_co()
    assert relerr(rg, ro) < 1e-12
    assert relerr(cg, co) < 1e-14


@pytest.mark.parametrize("name", CASES)
def test_jacobian_spmv_precondition(oracle_binding, gpu_binding, name):
    w, over = make(name)
    ho, hg = open_pair(oracle_binding, gpu_binding, w, **over)
    for h in (ho, hg):
        h.residual()
        h.assemble_jacobian()
    Do, Lo, Uo = ho.get_jacobian()
    Dg, Lg, Ug = hg.get_jacobian()
    assert relerr(Dg, Do) < 1e-12
    if len(Lo):
        assert relerr(Lg, Lo) < 1e-12
        assert relerr(Ug, Uo) < 1e-12
    x = np.random.default_rng(1).standard_normal((w.mesh.n_cells, 5))
    assert relerr(hg.matrix_mul(x), ho.matrix_mul(x)) < 1e-12
    assert relerr(hg.precondition(x), ho.precondition(x)) < 1e-12


@pytest.mark.parametrize("name", CASES)
def test_solve_and_update(oracle_binding, gpu_binding, name):
    w, over = make(name)
    ho, hg = open_pair(oracle_binding, gpu_binding, w, **over)
    for h in (ho, hg):
        h.residual()
        h.assemble_jacobian()
    po, dWo, _ = ho.solve_increment()
    pg, dWg, _ = hg.solve_increment()
    assert pg.n_iterations == po.n_iterations
    assert np.allclose(pg.init_res, po.init_res, rtol=1e-11, atol=1e-300)
    assert relerr(dWg, dWo) < 1e-10
    ho.update_fields()
    hg.update_fields()
    assert relerr(hg.get_state()["W"], ho.get_state()["W"]) < 1e-10
    bo, bg = ho.get_boundary_state(), hg.get_boundary_state()
    for k in ("p", "U", "T"):
        assert relerr(bg[k], bo[k]) < 1e-10


@pytest.mark.parametrize("name", ["tube_ausm_natural", "bump_hllc_muscl_colour", "box_ausm_rcm",
                                  "bump_hllc_muscl_colour_levels"])
def test_pseudo_trajectory(oracle_binding, gpu_binding, name):
    """Several full pseudo iterations (SER, local dtau, GMRES, update) in lockstep."""
    w = WORKLOADS[name]()
    if name.startswith("box"):
        w = perturb(w)  # a uniform stream is a fixed point (residual = round-off)
    ho, hg = open_pair(oracle_binding, gpu_binding, w)
    unsteady = w.settings.get("ddt_scheme", 0) != 0
    for it in range(6):
        if unsteady and it % 3 == 0:
            ho.begin_time_step()
            hg.begin_time_step()
        so = ho.pseudo_iteration()
        sg = hg.pseudo_iteration()
        assert sg.perf.n_iterations == so.perf.n_iterations
        assert abs(sg.rho_l2_residual - so.rho_l2_residual) <= 1e-10 * so.rho_l2_residual
        assert relerr(hg.get_state()["W"], ho.get_state()["W"]) < 1e-9


@pytest.mark.parametrize("name", ["bump_hllc_muscl_colour", "box_ausm_rcm"])
def test_mixed_precision(oracle_binding, gpu_binding, name):
    """FP32 Jacobian / preconditioner / Krylov basis under the FP64 residual."""
    w, _ = make(name)
    ho = cases_open(oracle_binding, w)
    hg = cases_open(gpu_binding, w, precision=1)
    for h in (ho, hg):
        h.residual()
        h.assemble_jacobian()
    Do, Lo, Uo = ho.get_jacobian()
    Dg, Lg, Ug = hg.get_jacobian()
    assert relerr(Dg, Do) < 1e-6
    assert relerr(Lg, Lo) < 1e-6
    _, dWo, _ = ho.solve_increment()
    _, dWg, _ = hg.solve_increment()
    assert relerr(dWg, dWo) < 5e-3
    ho.update_fields()
    hg.update_fields()
    assert relerr(hg.get_state()["W"], ho.get_state()["W"]) < 1e-4


def test_mixed_converges_like_fp64(gpu_binding):
    """Mixed and FP64 GPU runs reach the same steady state."""
    w = cases.bump_channel(24, 8, 4, ordering_mode="colour")
    res = {}
    for prec in (0, 1):
        h = cases_open(gpu_binding, w, precision=prec, pseudo_co_num_max=50.0)
        r0 = None
        for it in range(400):
            s = h.pseudo_iteration()
            r0 = r0 or s.rho_l2_residual
            if s.rho_l2_residual / r0 < 1e-9:
                break
        res[prec] = h.get_state()["W"]
    assert relerr(res[1], res[0]) < 1e-6


@pytest.mark.parametrize("precision,tol", [(0, 1e-12), (1, 1e-5)])
def test_sync_free_lusgs_sweeps(oracle_binding, gpu_binding, precision, tol):
    """Natural numbering of a 128x64x64 box: 254 levels of ~2,000 rows, swept
    by one sync-free launch per direction; identical to the sequential sweep."""
    w = cases.bump_channel(128, 64, 64, ordering_mode="natural", second_order=False)
    hg = cases_open(gpu_binding, w, precision=precision)
    ho = cases_open(oracle_binding, w)
    for h in (hg, ho):
        h.residual()
        h.assemble_jacobian()
    r = np.random.default_rng(4).standard_normal((w.mesh.n_cells, 5))
    assert relerr(hg.precondition(r), ho.precondition(r)) < tol
