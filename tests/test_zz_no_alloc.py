"""The allocation-free linear residual against the existing entry points (GPU).

``ics_linear_residual_noalloc`` serves callers that may not allocate device
memory while they run (real-time drivers that allocate only at start-up,
hosts that own every device buffer through their own pool): they pass device
buffers for x, r and the L1 sums, and the kernel's scratch is a fixed array
inside the library.  Its r = b - A x must equal the one built from the
existing entry points (b from ics_residual, A x from ics_matrix_mul), on two
calls in a row because the fixed array keeps the previous call's contents.
The cases cover the plain inviscid bump, the viscous box with the non-LF
viscous Jacobian (its extra per-slot laplacian terms) and an annular sector
with a rotating MRF zone (its skew source block), in both precisions.  This
file is collected last so a failure here leaves every other test already run.
"""

import numpy as np
import pytest

from icsfoam_gb300 import abi, cases

pytestmark = pytest.mark.gpu


def relerr(a, b):
    s = np.abs(b).max(axis=0)
    s[1:4] = s[1:4].max()
    return float((np.abs(a - b) / np.where(s == 0, 1.0, s)).max())


def _workload(b, name, precision):
    """(workload, handle) with a residual and an assembled Jacobian."""
    from icsfoam_gb300 import mrf as MRF

    import test_viscous_jacobian as tv

    if name == "bump":
        w = cases.bump_channel(24, 8, 4, ordering_mode="colour")
        over = {}
    elif name == "viscous_box":
        w = tv.workload("box")
        over = {"viscous_lf_jacobian": 0}
    else:
        from test_gpu_mrf import sector

        w = sector("HLLC")
        over = {}
    h = abi.CaseHandle(b, w.mesh, cases.make_config(b, w.settings, precision=precision, **over))
    h.set_primitive(w.p, w.U, w.T)
    if name == "mrf_sector":
        h.set_mrf(MRF.frame_fields(w.mesh, *w.mrf), 0)
    return w, h


@pytest.mark.parametrize("name", ["bump", "viscous_box", "mrf_sector"])
@pytest.mark.parametrize("precision,tol", [(0, 1e-12), (1, 1e-5)])
def test_noalloc_matches_existing_entry_points(gpu_binding, name, precision, tol):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    w, h = _workload(gpu_binding, name, precision)
    b = h.residual()
    h.assemble_jacobian()
    rng = np.random.default_rng(7)
    for call in range(2):
        x = rng.standard_normal((w.mesh.n_cells, 5)) * np.array([1.0, 100.0, 100.0, 100.0, 1e5])
        ref = b - h.matrix_mul(x)
        xd = torch.tensor(x, dtype=torch.float64, device="cuda")
        rd = torch.full_like(xd, float("nan"))
        l1 = torch.full((5,), float("nan"), dtype=torch.float64, device="cuda")
        # x is written on torch's stream; the call runs on the handle's stream
        torch.cuda.synchronize()
        st = h.linear_residual_noalloc(xd.data_ptr(), rd.data_ptr(), l1.data_ptr())
        assert st == abi.ICS_OK, call
        r = rd.cpu().numpy()
        assert relerr(r, ref) < tol, call
        assert np.allclose(l1.cpu().numpy(), np.abs(ref).sum(axis=0), rtol=tol, atol=0), call


def test_noalloc_rejects_cases_beyond_its_scratch(gpu_binding):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    n = 2_097_152 + 1
    w = cases.shock_tube(n, ordering_mode="colour")
    h = abi.CaseHandle(gpu_binding, w.mesh, cases.make_config(gpu_binding, w.settings))
    h.set_primitive(w.p, w.U, w.T)
    h.begin_time_step()
    h.residual()
    h.assemble_jacobian()
    xd = torch.zeros((n, 5), dtype=torch.float64, device="cuda")
    rd = torch.zeros_like(xd)
    l1 = torch.zeros(5, dtype=torch.float64, device="cuda")
    assert h.linear_residual_noalloc(xd.data_ptr(), rd.data_ptr(), l1.data_ptr()) == abi.ICS_ERR_ARG
