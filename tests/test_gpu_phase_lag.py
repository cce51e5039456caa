"""Phase-lag cyclic patches (Harmonic Balance) on the CUDA path.

The 20-degree sector stacked into 3 instances with its cyclic pair
phase-lagged (with and without cylindrical velocity): residual, Jacobian and
pseudo iterations against the oracle; the travelling-wave known answer
against the 40-degree sector on the GPU; the residual's tangent against
finite differences of the oracle (the instances couple through the
phase-lagged neighbours) and the exact Jacobian built from it.
"""

import numpy as np
import pytest

from icsfoam_gb300 import abi, cases
from icsfoam_gb300 import hb as HB

from test_cyclic import _rows  # noqa: E402
from test_gpu_diff import direction, fd_jvp  # noqa: E402
from test_gpu_parity import relerr  # noqa: E402
from test_phase_lag import FREQ, _open, _stack, _wave  # noqa: E402

pytestmark = pytest.mark.gpu


def _case(flux="HLLC", cyl=False, ibpa=0.7, seed=4):
    base = cases.annular_sector(5, 6, 6, ordering_mode="colour", flux=flux)
    n = 3
    om = HB.omega_list([FREQ], [1])
    t = HB.select_instants(om, n, None)
    st, D = _stack(base, n, om, t)
    rng = np.random.default_rng(seed)
    N = st.n_cells
    p = np.concatenate([base.p] * n) * (1 + 0.02 * rng.uniform(-1, 1, N))
    T = np.concatenate([base.T] * n) * (1 + 0.02 * rng.uniform(-1, 1, N))
    U = np.concatenate([base.U] * n) + rng.uniform(-4, 4, (N, 3))
    plag = HB.phase_lag_setup(st, n, om, t, ibpa, cyl_coords=cyl)
    return base, st, (n, D), p, U, T, plag


@pytest.mark.parametrize("flux,cyl", [("HLLC", False), ("HLLC", True), ("AUSMPlusUp", True), ("ROE", False)])
def test_phase_lag_residual_jacobian_and_iterations(gpu_binding, oracle_binding, flux, cyl):
    base, st, hbop, p, U, T, plag = _case(flux, cyl)
    hg = _open(gpu_binding, st, base.settings, hbop, p, U, T, plag)
    ho = _open(oracle_binding, st, base.settings, hbop, p, U, T, plag)
    bg, bo = hg.get_boundary_state(), ho.get_boundary_state()
    assert relerr(bg["U"], bo["U"]) < 1e-14 and relerr(bg["p"], bo["p"]) < 1e-14
    assert relerr(hg.residual(), ho.residual()) < 1e-12
    assert relerr(hg.get_pseudo_co()[1], ho.get_pseudo_co()[1]) < 1e-12
    for h in (hg, ho):
        h.assemble_jacobian()
    assert relerr(hg.get_jacobian()[0], ho.get_jacobian()[0]) < 1e-12
    x = np.random.default_rng(1).standard_normal((st.n_cells, 5))
    assert relerr(hg.matrix_mul(x), ho.matrix_mul(x)) < 1e-12
    for it in range(3):
        hg.pseudo_iteration()
        ho.pseudo_iteration()
        assert relerr(hg.get_state()["W"], ho.get_state()["W"]) < 1e-10, it


def test_travelling_wave_known_answer_on_gpu(gpu_binding):
    n, ibpa = 3, 0.6
    om = HB.omega_list([FREQ], [1])
    t = HB.select_instants(om, n, None)
    wa = cases.annular_sector(4, 6, 5, sector_deg=20.0, ordering_mode="natural", second_order=False)
    wb = cases.annular_sector(4, 12, 5, sector_deg=40.0, theta0_deg=-10.0, ordering_mode="natural",
                              second_order=False)
    k = ibpa / np.radians(20.0)
    res = []
    for w, phase in ((wa, ibpa), (wb, 2 * ibpa)):
        st, D = _stack(w, n, om, t)
        N = st.n_cells
        U = np.zeros((N, 3))
        U[:, 2] = 120.0
        h = _open(gpu_binding, st, w.settings, (n, D), _wave(w.mesh, n, t, k), U, np.full(N, 285.0),
                  HB.phase_lag_setup(st, n, om, t, phase))
        res.append(h.residual())
    rows = _rows(wa.mesh, wb.mesh)
    rows_all = np.concatenate([J * wb.mesh.n_cells + rows for J in range(n)])
    assert relerr(res[1][rows_all], res[0]) < 1e-9


def test_phase_lag_tangent_and_exact_jacobian(gpu_binding, oracle_binding):
    base, st, hbop, p, U, T, plag = _case("HLLC", True)
    hs = [_open(b, st, base.settings, hbop, p, U, T, plag) for b in (gpu_binding, oracle_binding)]
    bs = hs[0].get_boundary_state()
    rng = np.random.default_rng(5)
    B = len(bs["p"])
    pb = bs["p"] * (1 + 0.01 * rng.uniform(-1, 1, B))
    Tb = bs["T"] * (1 + 0.01 * rng.uniform(-1, 1, B))
    Ub = bs["U"] + rng.uniform(-1, 1, (B, 3))
    for h in hs:
        h.set_boundary_state(pb, Ub, Tb, bs["phi"])
    hg, ho = hs
    W = hg.get_state()["W"]
    for seed in range(2):
        v = direction(W, seed)
        assert relerr(hg.jvp(v), fd_jvp(ho, W, v)) < 1e-5, seed
    hg.assemble_exact_jacobian()
    ptr, cols, blocks = hg.get_exact_jacobian()
    N = st.n_cells
    v = direction(W, 9)
    rows = np.repeat(np.arange(N), np.diff(ptr))
    jv = np.zeros((N, 5))
    np.add.at(jv, rows, np.einsum("jik,jk->ji", blocks, v[cols]))
    assert relerr(jv, hg.jvp(v)) < 1e-11
