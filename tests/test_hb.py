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
