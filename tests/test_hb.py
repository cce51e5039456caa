"""Harmonic Balance: spectral operator, instants and the oracle's coupling.

The operator is checked through properties the reference's construction
implies (HBZone.C:270-356): D applied to samples of any signal band-limited
to the omega list returns its time derivative at the instants, D annihilates
constants, and the period search returns the best-conditioned period.  The
oracle's coupling terms are checked against the same stacked case without
HB: the residual source differs by -V (D x I) W and the matrix action by
V (D x I) x.  With identical instances the HB solution is the steady one.
"""

import numpy as np
import pytest

from icsfoam_gb300 import abi, cases, hb as HB


def test_omega_list_order():
    om = HB.omega_list([10.0, -3.0], [2, 1])
    assert list(om) == [0.0, 10.0, 20.0, 3.0, -3.0, -20.0, -10.0]
    with pytest.raises(ValueError):
        HB.omega_list([1.0], [1, 2])


@pytest.mark.parametrize("H,selected", [(1, True), (2, True), (1, False), (3, False)])
def test_operator_differentiates_band_limited_signals(H, selected):
    w0 = 2 * np.pi * 7.0
    om = HB.omega_list([w0], [H])
    n = 2 * H + 1
    t = HB.select_instants(om, n, 2 * np.pi / w0 if selected else None)
    D = HB.hb_operator(om, t)
    rng = np.random.default_rng(H)
    a, b = rng.standard_normal(H + 1), rng.standard_normal(H + 1)
    f = a[0] + sum(a[k] * np.cos(k * w0 * t) + b[k] * np.sin(k * w0 * t) for k in range(1, H + 1))
    df = sum(-a[k] * k * w0 * np.sin(k * w0 * t) + b[k] * k * w0 * np.cos(k * w0 * t) for k in range(1, H + 1))
    assert np.abs(D @ f - df).max() < 1e-10 * w0 * H
    assert np.abs(D.sum(axis=1)).max() < 1e-10 * w0 * H
    if selected:
        # equispaced over the true period: antisymmetric, zero diagonal
        assert np.abs(D + D.T).max() < 1e-10 * w0 * H


def test_period_search_picks_best_conditioned_period():
    om = HB.omega_list([3.0, 5.0], [1, 1])
    n = 5
    t = HB.select_instants(om, n)
    T = t[1] * n
    T0 = HB.find_t0(om)
    assert T0 <= T <= 5.0 * T0 + 1e-3 * T0
    best = HB.condition_number(om, t)
    for frac in (1.0, 1.37, 2.0, 3.1, 4.9):
        other = (frac * T0 / n) * np.arange(n)
        assert best <= HB.condition_number(om, other) + 1e-12


def eq_scale(*arrs):
    """Per-equation max-norm (momentum components share one), never zero."""
    m = sum(np.abs(a).max(axis=0) for a in arrs)
    m[1:4] = m[1:4].max()
    return np.where(m == 0, 1.0, m)


def stacked(w, n, D):
    st = HB.stack_instances(w.mesh, n)
    rep = lambda a: np.concatenate([a] * n)
    return cases.Workload(w.name, st, rep(w.p), rep(w.U), rep(w.T), dict(w.settings), hb=(n, D))


def open_case(b, w, hb=True, **over):
    h = abi.CaseHandle(b, w.mesh, cases.make_config(b, w.settings, **over))
    if hb and w.hb:
        h.set_hb(*w.hb)
    h.set_primitive(w.p, w.U, w.T)
    return h


def test_coupling_terms_in_source_and_matrix_action(oracle_binding):
    w = cases.hb_bump_channel(12, 4, 2, amplitude=0.1)
    n, D = w.hb
    hh, h1 = open_case(oracle_binding, w), open_case(oracle_binding, w, hb=False)
    s_hb, s_1 = hh.residual(), h1.residual()
    W = hh.get_state()["W"]
    Nc = w.mesh.n_cells // n
    V = w.mesh.V
    Wi = W.reshape(n, Nc, 5)
    expect = -(V.reshape(n, Nc)[..., None] * np.einsum("jk,kcq->jcq", D, Wi)).reshape(-1, 5)
    scale = eq_scale(s_1, expect)
    assert (np.abs((s_hb - s_1) - expect) / scale).max() < 1e-12
    hh.assemble_jacobian()
    h1.assemble_jacobian()
    x = np.random.default_rng(0).standard_normal((w.mesh.n_cells, 5))
    y_hb, y_1 = hh.matrix_mul(x), h1.matrix_mul(x)
    xi = x.reshape(n, Nc, 5)
    expect = (V.reshape(n, Nc)[..., None] * np.einsum("jk,kcq->jcq", D, xi)).reshape(-1, 5)
    scale = eq_scale(y_1)
    assert (np.abs((y_hb - y_1) - expect) / scale).max() < 1e-12


@pytest.mark.parametrize("second_order,tol", [(False, 1e-12), (True, 1e-5)])
def test_identical_instances_follow_the_steady_solution(oracle_binding, second_order, tol):
    """D annihilates constants: stacked identical instances iterate like one.

    First order the trajectories agree to round-off; with the limited MUSCL
    reconstruction the limiter's switches amplify the round-off of the
    (zero-row-sum) coupling, so the bound is looser.
    """
    w = cases.bump_channel(12, 4, 2, ordering_mode="colour", second_order=second_order)
    om = HB.omega_list([50.0], [1])
    D = HB.hb_operator(om, HB.select_instants(om, 3, 2 * np.pi / 50.0))
    hs = open_case(oracle_binding, w)
    hh = open_case(oracle_binding, stacked(w, 3, D))
    for _ in range(5):
        hs.pseudo_iteration()
        hh.pseudo_iteration()
    Ws = hs.get_state()["W"]
    Wh = hh.get_state()["W"].reshape(3, -1, 5)
    for J in range(3):
        assert np.abs(Wh[J] - Ws).max() / np.abs(Ws).max() < tol


def test_time_periodic_case_converges_per_instance(oracle_binding):
    w = cases.hb_bump_channel(12, 4, 2, amplitude=0.1, second_order=False)
    h = open_case(oracle_binding, w, pseudo_co_num_max=50.0)
    r = []
    for _ in range(48):
        s = h.pseudo_iteration()
        r.append(max(s.perf.init_res))
    assert r[-1] < 2e-2 * r[0]
    # the instances see different back pressures: their states differ
    W = h.get_state()["W"].reshape(3, -1, 5)
    assert np.abs(W[0, :, 0] - W[1, :, 0]).max() > 1e-4 * np.abs(W[0, :, 0]).max()


def test_errors(oracle_binding):
    w = cases.hb_bump_channel(8, 4, 2)
    n, D = w.hb
    h = open_case(oracle_binding, w, hb=False)
    assert w.mesh.n_cells % 5 != 0
    with pytest.raises(abi.IcsError) as e:
        h.set_hb(5, np.zeros((5, 5)))
    assert e.value.status == abi.ICS_ERR_ARG
    h.set_hb(n, D)
    cfg = cases.make_config(oracle_binding, w.settings, solver=1)
    with pytest.raises(abi.IcsError) as e:
        h.set_config(cfg)
    assert e.value.status == abi.ICS_ERR_ARG
    h2 = open_case(oracle_binding, w, hb=False, ddt_scheme=1)
    with pytest.raises(abi.IcsError) as e:
        h2.set_hb(n, D)
    assert e.value.status == abi.ICS_ERR_ARG
    with pytest.raises(abi.IcsError):
        h.set_hb(17, np.zeros((17, 17)))


@pytest.mark.parametrize("H,selected", [(1, True), (2, False)])
def test_reconstruction_recovers_band_limited_history(H, selected):
    """reconstructHBFoam: the snapshots of a band-limited history give it back at any time."""
    w0 = 2 * np.pi * 3.0
    om = HB.omega_list([w0], [H])
    t = HB.select_instants(om, 2 * H + 1, 2 * np.pi / w0 if selected else None)
    rng = np.random.default_rng(5)
    a, b = rng.standard_normal((H + 1, 4)), rng.standard_normal((H + 1, 4))

    def f(tt):
        return a[0] + sum(a[k] * np.cos(k * w0 * tt) + b[k] * np.sin(k * w0 * tt) for k in range(1, H + 1))

    snaps = np.stack([f(tj) for tj in t])
    for tt in (0.0137, 0.2, 1.7):
        assert np.allclose(HB.reconstruct(om, t, snaps, tt), f(tt), atol=1e-10)
    # at an instant the weights select that snapshot
    assert np.allclose(HB.reconstruction_weights(om, t, t[1]), np.eye(2 * H + 1)[1], atol=1e-10)


def _zone_case():
    """HB annular sector (slip sides) whose instance meshes are rotated about
    the axis by different angles, so that the cylindrical frames of the
    instances differ; zone: the upstream half of the cells."""
    w = cases.hb_annular_sector(4, 6, 6, harmonics=1, sides="slip")
    m = w.mesh
    n, D = w.hb
    Nc = m.n_cells // n
    rng = np.random.default_rng(8)
    w.p = w.p * (1 + 0.02 * rng.uniform(-1, 1, m.n_cells))
    w.U = w.U + 5.0 * rng.uniform(-1, 1, (m.n_cells, 3))

    def rot(a):
        c, s = np.cos(a), np.sin(a)
        return np.array([[c, -s, 0.0], [s, c, 0.0], [0.0, 0.0, 1.0]])

    inst_f = m.owner // Nc
    inst_b = m.b_cell // Nc
    for K in range(n):
        R = rot(0.05 * K)
        m.C[K * Nc:(K + 1) * Nc] = m.C[K * Nc:(K + 1) * Nc] @ R.T
        for a in (m.Sf, m.Cf):
            a[inst_f == K] = a[inst_f == K] @ R.T
        for a in (m.b_Sf, m.b_Cf):
            a[inst_b == K] = a[inst_b == K] @ R.T
        w.U[K * Nc:(K + 1) * Nc] = w.U[K * Nc:(K + 1) * Nc] @ R.T
    zone = (m.C[:Nc, 2] < 0.1).astype(np.int32)
    return w, zone


def test_hb_zone_and_cylindrical_source(oracle_binding):
    """The HB zone carries the source and couplings, the other cells neither;
    every cell as the zone is the default; with identical instance frames the
    cylindrical combination equals the Cartesian one; with rotated instances
    it differs only in the momentum source, and the Jacobian stays Cartesian
    (HBZone.C:435-519)."""
    w, zone = _zone_case()
    n, D = w.hb
    Nc = w.mesh.n_cells // n

    def opened(zone_=None, cyl=False, Dm=D):
        h = abi.CaseHandle(oracle_binding, w.mesh, cases.make_config(oracle_binding, w.settings))
        h.set_hb(n, Dm)
        h.set_primitive(w.p, w.U, w.T)
        if zone_ is not None or cyl:
            h.set_hb_zone(zone_, cyl, (0.0, 0.0, 1.0), (0.0, 0.0, 0.0))
        return h

    base = opened()
    r0 = base.residual()
    base.assemble_jacobian()
    x = np.random.default_rng(2).standard_normal((w.mesh.n_cells, 5))
    y0 = base.matrix_mul(x)
    every = opened(np.ones(Nc, np.int32))
    assert np.array_equal(every.residual(), r0)
    every.assemble_jacobian()
    assert np.array_equal(every.matrix_mul(x), y0)
    # outside the zone: the residual and matrix action of uncoupled instances
    zoned = opened(zone)
    free = opened(Dm=np.zeros_like(D))
    rz, rf = zoned.residual(), free.residual()
    out = np.tile(zone == 0, n)
    assert np.array_equal(rz[out], rf[out]) and np.array_equal(rz[~out], r0[~out])
    zoned.assemble_jacobian()
    free.assemble_jacobian()
    yz, yf = zoned.matrix_mul(x), free.matrix_mul(x)
    assert np.allclose(yz[out], yf[out], rtol=1e-14, atol=0) and np.allclose(yz[~out], y0[~out], rtol=1e-14, atol=0)
    # cylindrical components: only the momentum source changes, the matrix does not
    cyl = opened(cyl=True)
    rc = cyl.residual()
    assert np.array_equal(rc[:, [0, 4]], r0[:, [0, 4]])
    assert not np.allclose(rc[:, 1:4], r0[:, 1:4], rtol=1e-9, atol=0)
    cyl.assemble_jacobian()
    assert np.allclose(cyl.matrix_mul(x), y0, rtol=1e-14, atol=1e-300)
    # identical instance meshes: the cylindrical frames agree and the two
    # combinations give the same source up to round-off
    w2 = cases.hb_annular_sector(4, 6, 6, harmonics=1, sides="slip")
    w2.U = w.U
    res = []
    for c in (False, True):
        h = abi.CaseHandle(oracle_binding, w2.mesh, cases.make_config(oracle_binding, w2.settings))
        h.set_hb(*w2.hb)
        h.set_primitive(w.p, w.U, w.T)
        if c:
            h.set_hb_zone(None, True, (0.0, 0.0, 1.0), (0.0, 0.0, 0.0))
        res.append(h.residual())
    scale = np.abs(res[0]).max(axis=0)
    assert np.max(np.abs(res[1] - res[0]) / scale) < 1e-12
