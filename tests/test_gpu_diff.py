"""Differentiation of the residual on the CUDA path.

The Jacobian-vector product (forward-mode dual numbers through the residual
kernels) is checked against central finite differences of the ORACLE's
residual, h = 1e-8 relative to each equation's state scale, along seeded
directions; the exact Jacobian assembled from coloured products must
reproduce the same product, and its transpose product must satisfy
<u, J v> = <J^T u, v>.

The discrete residual is only piecewise smooth.  Interior states are
randomly perturbed, and so are the (fixed) boundary values: right after
ics_set_primitive a zeroGradient or slip boundary value equals its cell's
value exactly, which puts the limiters' max/min selections at a tie where
the residual has no derivative (central differences then average the two
one-sided slopes while the JVP follows the branch the comparison selects).

Tolerances: JVP vs FD 1e-5 of each equation's max |J v| (FD round-off is
~1e-16 of the face fluxes / 1e-8); exact blocks vs JVP and the adjoint
identity 1e-11.
"""

import numpy as np
import pytest

from icsfoam_gb300 import abi, cases

from test_gpu_parity import perturb, relerr  # noqa: E402

pytestmark = pytest.mark.gpu

WORKLOADS = {
    "tube_ausm": lambda: cases.shock_tube(60),
    "bump_hllc_muscl": lambda: cases.bump_channel(12, 6, 3, ordering_mode="colour", flux="HLLC"),
    "bump_ausm_muscl_minmod": lambda: _over(cases.bump_channel(10, 5, 3, ordering_mode="colour", flux="AUSMPlusUp"),
                                            recon_rho=4, recon_U=4, recon_T=4),
    "bump_roe_vanleer": lambda: _over(cases.bump_channel(10, 5, 3, ordering_mode="natural", flux="ROE"),
                                      recon_rho=1, recon_U=1, recon_T=1),
    "box_viscous_ausm": lambda: cases.random_box(5),
    "hb_bump_hllc": lambda: cases.hb_bump_channel(8, 4, 2, amplitude=0.1),
}


def _over(w, **kw):
    w.settings = dict(w.settings, **kw)
    return w


def open_case(b, w, untie=True):
    h = abi.CaseHandle(b, w.mesh, cases.make_config(b, w.settings))
    if w.hb:
        h.set_hb(*w.hb)
    h.set_primitive(w.p, w.U, w.T)
    if untie:
        bs = h.get_boundary_state()
        rng = np.random.default_rng(5)
        B = len(bs["p"])
        p = bs["p"] * (1 + 0.01 * rng.uniform(-1, 1, B))
        T = bs["T"] * (1 + 0.01 * rng.uniform(-1, 1, B))
        U = bs["U"] + rng.uniform(-1, 1, (B, 3))
        h.set_boundary_state(p, U, T, bs["phi"])
    return h


def fd_jvp(h, W, v, eps=1e-8):
    h.set_conservative(W + eps * v)
    rp = h.residual()
    h.set_conservative(W - eps * v)
    rm = h.residual()
    h.set_conservative(W)
    return (rp - rm) / (2 * eps)


def direction(W, seed):
    rng = np.random.default_rng(seed)
    scale = np.abs(W).max(axis=0)
    scale[1:4] = scale[1:4].max()
    return rng.standard_normal(W.shape) * scale


@pytest.mark.parametrize("name", list(WORKLOADS))
def test_jvp_matches_oracle_finite_differences(gpu_binding, oracle_binding, name):
    w = perturb(WORKLOADS[name]())
    hg, ho = open_case(gpu_binding, w), open_case(oracle_binding, w)
    W = hg.get_state()["W"]
    for seed in range(3):
        v = direction(W, seed)
        jv = hg.jvp(v)
        fd = fd_jvp(ho, W, v)
        assert relerr(jv, fd) < 1e-5, (name, seed)


@pytest.mark.parametrize("name", ["bump_hllc_muscl", "box_viscous_ausm", "hb_bump_hllc"])
def test_exact_jacobian_and_transpose_product(gpu_binding, name):
    w = perturb(WORKLOADS[name]())
    h = open_case(gpu_binding, w)
    nnz, ncol = h.assemble_exact_jacobian()
    assert 0 < ncol <= 80 * (w.hb[0] if w.hb else 1)
    ptr, cols, blocks = h.get_exact_jacobian()
    assert ptr[-1] == nnz
    W = h.get_state()["W"]
    N = w.mesh.n_cells
    rng = np.random.default_rng(7)
    for seed in range(2):
        v = direction(W, 10 + seed)
        jv = h.jvp(v)
        rows = np.repeat(np.arange(N), np.diff(ptr))
        jv_csr = np.zeros((N, 5))
        np.add.at(jv_csr, rows, np.einsum("jik,jk->ji", blocks, v[cols]))
        assert relerr(jv_csr, jv) < 1e-11
        u = rng.standard_normal((N, 5))
        jtu = h.vjp(u)
        lhs, rhs = float(np.sum(u * jv)), float(np.sum(jtu * v))
        assert abs(lhs - rhs) <= 1e-11 * (np.abs(u * jv).sum() + np.abs(jtu * v).sum())
    # the same product through the transpose gather and a dense restatement
    J = np.zeros((5 * N, 5 * N))
    for r in range(N):
        for j in range(ptr[r], ptr[r + 1]):
            J[5 * r:5 * r + 5, 5 * cols[j]:5 * cols[j] + 5] = blocks[j]
    u = rng.standard_normal((N, 5))
    assert relerr(h.vjp(u), (J.T @ u.reshape(-1)).reshape(N, 5)) < 1e-12


def test_exact_jacobian_invalidated_by_state_change(gpu_binding):
    w = perturb(WORKLOADS["bump_hllc_muscl"]())
    h = open_case(gpu_binding, w)
    h.assemble_exact_jacobian()
    h.get_exact_jacobian()
    W = h.get_state()["W"]
    h.set_conservative(W * 1.01)
    with pytest.raises(abi.IcsError) as e:
        h.get_exact_jacobian()
    assert e.value.status == abi.ICS_ERR_STATE
    # vjp reassembles at the new state
    u = np.random.default_rng(3).standard_normal(W.shape)
    v = direction(W, 4)
    assert abs(np.sum(u * h.jvp(v)) - np.sum(h.vjp(u) * v)) < 1e-10 * np.abs(u * h.jvp(v)).sum()


def test_swept_bump_32_directions(gpu_binding, oracle_binding):
    """The differentiation workload (30-degree swept 8% bump, M 0.84, 3 degrees
    incidence, HLLC + MUSCL/Venkatakrishnan) at a small size: JVP along 32
    seeded directions against the oracle's central differences."""
    w = perturb(cases.swept_bump(12, 6, 4))
    hg, ho = open_case(gpu_binding, w), open_case(oracle_binding, w)
    W = hg.get_state()["W"]
    worst = 0.0
    for s in range(32):
        v = direction(W, 100 + s)
        worst = max(worst, relerr(hg.jvp(v), fd_jvp(ho, W, v)))
    assert worst < 1e-5


def test_swept_bump_full_size_derivatives(gpu_binding):
    """The differentiation workload at its configured size, 240x128x128
    (3,932,160 cells), on a perturbed state with the boundary values untied
    from the cells (a zeroGradient boundary value equal to its cell's is a
    tie of the limiter's bounds, where the residual has no derivative):
      * along 32 seeded directions the JVP equals central differences with the
        step 1e-7 to 1e-5 of each equation's max-norm at every cell where the
        residual is smooth over the step (the forward and backward differences
        agree to 1e-6: |R(W+hv) - 2 R(W) + R(W-hv)| / h), and at all but 1% of
        all cells; the 2-norm of the difference stays below 1e-2 of the FD's.
        The cells above 1e-5 lie within a step of a kink of the limiters'
        min / max selections or of Venkatakrishnan's steep ratio, where the
        one-sided derivative of the JVP and the average slope of a central
        difference differ;
      * the reverse-mode VJP (gradients recomputed) is the JVP's transpose,
        <u, J v> = <J^T u, v> to 1e-12 of |u| |J v|, and equals the product
        with the assembled exact Jacobian (97 M stencil blocks) to 1e-10."""
    w = perturb(cases.swept_bump(240, 128, 128))
    h = open_case(gpu_binding, w, untie=True)
    W = h.get_state()["W"]
    R0 = h.residual()
    eps = 1e-7
    over = 0
    for s in range(32):
        v = direction(W, 100 + s)
        J = h.jvp(v)
        h.set_conservative(W + eps * v)
        Rp = h.residual()
        h.set_conservative(W - eps * v)
        Rm = h.residual()
        h.set_conservative(W)
        F = (Rp - Rm) / (2 * eps)
        scale = np.abs(F).max(axis=0)
        scale[1:4] = scale[1:4].max()
        err = (np.abs(J - F) / scale).max(axis=1)
        smooth = (np.abs(Rp - 2 * R0 + Rm) / eps / scale).max(axis=1) < 1e-6
        assert smooth.sum() > 0.01 * W.shape[0] and err[smooth].max() < 1e-5, (s, err[smooth].max())
        assert np.linalg.norm(J - F) < 1e-2 * np.linalg.norm(F), s
        over += int((err > 1e-5).sum())
    assert over < 0.01 * 32 * W.shape[0], over
    rng = np.random.default_rng(7)
    for s in range(4):
        u = rng.standard_normal(W.shape)
        v = direction(W, 200 + s)
        Jv = h.jvp(v)
        assert abs(np.sum(u * Jv) - np.sum(h.vjp_recompute(u) * v)) <= 1e-12 * np.linalg.norm(u) * np.linalg.norm(Jv)
    h.assemble_exact_jacobian()
    for s in range(2):
        u = rng.standard_normal(W.shape)
        assert relerr(h.vjp_recompute(u), h.vjp(u)) < 1e-10


def test_torch_autograd_backward_is_the_exact_vjp(gpu_binding):
    import torch

    from icsfoam_gb300 import autograd

    w = perturb(WORKLOADS["bump_hllc_muscl"]())
    h = open_case(gpu_binding, w)
    W0 = h.get_state()["W"]
    W = torch.tensor(W0, device="cuda", requires_grad=True)
    g = torch.randn(W.shape, dtype=torch.float64, device="cuda", generator=torch.Generator("cuda").manual_seed(0))
    R = autograd.residual(h, W)
    assert relerr(R.detach().cpu().numpy(), h.residual()) < 1e-14
    (R * g).sum().backward()
    expect = h.vjp(g.cpu().numpy())
    assert relerr(W.grad.cpu().numpy(), expect) < 1e-13
    v = torch.tensor(direction(W0, 3), device="cuda")
    assert relerr(autograd.jvp(h, W.detach(), v).cpu().numpy(), h.jvp(v.cpu().numpy())) < 1e-13
