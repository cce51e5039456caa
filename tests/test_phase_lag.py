"""Phase-lag cyclic patches of Harmonic Balance cases (CPU, the oracle).

* the operator: P(0) = I, P(a) P(b) = P(a + b), and P(a) applied to the
  instants of a band-limited signal gives the signal shifted by a/omega;
* with IBPA = 0 a phase-lag pair is the plain cyclic pair (residual and
  pseudo iterations);
* the known answer: a pressure wave travelling around the annulus, f(theta,
  t) = cos(omega t - (IBPA/Theta) theta), in a 20-degree sector whose cyclic
  pair is phase-lagged by IBPA, gives the residual of the 40-degree sector
  (phase lag 2 IBPA) in the same cells and instances -- the phase-lagged
  neighbour values are the travelling wave's continuation.  First-order
  reconstruction: the reference combines the instances for the fields only,
  the partner's gradients stay those of the face's own instance.
"""

import numpy as np
import pytest

from icsfoam_gb300 import abi, cases
from icsfoam_gb300 import hb as HB

from test_cyclic import _rows  # noqa: E402

FREQ = 50.0


def test_phase_lag_operator():
    om = HB.omega_list([FREQ], [2])
    t = HB.select_instants(om, 5, None)
    assert np.abs(HB.phase_lag_operator(om, t, 0.0) - np.eye(5)).max() < 1e-14
    Pa, Pb = HB.phase_lag_operator(om, t, 0.3), HB.phase_lag_operator(om, t, 0.5)
    assert np.abs(Pa @ Pb - HB.phase_lag_operator(om, t, 0.8)).max() < 1e-13
    w = FREQ  # omega_list takes angular frequencies
    f = 1.0 + 0.3 * np.cos(w * t + 0.2) - 0.1 * np.sin(2 * w * t)
    shifted = 1.0 + 0.3 * np.cos(w * t + 0.2 + 0.7) - 0.1 * np.sin(2 * (w * t + 0.7))
    assert np.abs(HB.phase_lag_operator(om, t, 0.7) @ f - shifted).max() < 1e-13


def _stack(base, n, omegas, instants):
    st = HB.stack_instances(base.mesh, n)
    D = HB.hb_operator(omegas, instants)
    return st, D


def _open(b, mesh, settings, hbop, p, U, T, plag=None):
    h = abi.CaseHandle(b, mesh, cases.make_config(b, settings))
    h.set_hb(*hbop)
    h.set_primitive(p, U, T)
    if plag is not None:
        h.set_phase_lag(plag)
    return h


@pytest.mark.parametrize("geometry,mode_cyl", [("translational", False), ("translational", True),
                                               ("rotational", False), ("rotational", True)])
def test_zero_ibpa_is_the_plain_cyclic(oracle_binding, geometry, mode_cyl):
    """IBPA = 0 makes P the identity: the phase-lag patch is the plain cyclic
    one (MUSCL, residual and two pseudo iterations).  Rotational pairs are
    compared on an axial velocity and one residual: the reference combines
    the velocity unrotated without cylCoords and rotated with them, where the
    plain cyclic patch rotates the vector and not its components."""
    from test_cyclic import _bump, _periodic_state
    n = 3
    om = HB.omega_list([FREQ], [1])
    t = HB.select_instants(om, n, None)
    if geometry == "translational":
        m = _bump(3, 0.3)
        base = cases.Workload("bump", m, *_periodic_state(m, 0.3), dict(cases.bump_channel(4, 2, 2).settings))
    else:
        base = cases.annular_sector(4, 6, 5, ordering_mode="colour")
    st, D = _stack(base, n, om, t)
    rng = np.random.default_rng(4)
    N = st.n_cells
    p = np.concatenate([base.p] * n) * (1 + 0.02 * rng.uniform(-1, 1, N))
    T = np.concatenate([base.T] * n) * (1 + 0.02 * rng.uniform(-1, 1, N))
    U = np.concatenate([base.U] * n)
    if geometry == "translational":
        U = U + rng.uniform(-3, 3, (N, 3))
    else:
        U[:, 2] += rng.uniform(-3, 3, N)
    h0 = _open(oracle_binding, st, base.settings, (n, D), p, U, T)
    h1 = _open(oracle_binding, st, base.settings, (n, D), p, U, T,
               HB.phase_lag_setup(st, n, om, t, 0.0, cyl_coords=mode_cyl))
    r0, r1 = h0.residual(), h1.residual()
    assert np.abs(r1 - r0).max() <= 1e-12 * np.abs(r0).max()
    if geometry == "rotational":
        return  # the first update gives the velocity components that tell the two apart
    for _ in range(2):
        h0.pseudo_iteration()
        h1.pseudo_iteration()
    W0, W1 = h0.get_state()["W"], h1.get_state()["W"]
    assert np.abs(W1 - W0).max() <= 1e-10 * np.abs(W0).max()


def _wave(mesh, n, instants, k):
    x, y, z = mesh.C.T
    th = np.arctan2(y, x)
    r = np.hypot(x, y)
    w = FREQ  # omega_list takes angular frequencies
    p = np.concatenate([8.5e4 * (1 + 0.04 * np.cos(w * tj - k * th + 3 * z + 2 * r)) for tj in instants])
    return p


@pytest.mark.parametrize("flux", ["HLLC", "AUSMPlusUp", "ROE"])
def test_phase_lag_equals_the_doubled_sector(oracle_binding, flux):
    n, ibpa = 3, 0.6
    om = HB.omega_list([FREQ], [1])
    t = HB.select_instants(om, n, None)
    wa = cases.annular_sector(4, 6, 5, sector_deg=20.0, ordering_mode="natural", flux=flux, second_order=False)
    wb = cases.annular_sector(4, 12, 5, sector_deg=40.0, theta0_deg=-10.0, ordering_mode="natural", flux=flux,
                              second_order=False)
    k = ibpa / np.radians(20.0)
    out = []
    for w, phase in ((wa, ibpa), (wb, 2 * ibpa)):
        st, D = _stack(w, n, om, t)
        N = st.n_cells
        p = _wave(w.mesh, n, t, k)
        T = np.full(N, 285.0)
        U = np.zeros((N, 3))
        U[:, 2] = 120.0
        h = _open(oracle_binding, st, w.settings, (n, D), p, U, T, HB.phase_lag_setup(st, n, om, t, phase))
        out.append((st, h.residual(), w.mesh.n_cells))
    (sa, ra, Na), (sb, rb, Nb) = out
    rows = _rows(wa.mesh, wb.mesh)
    rows_all = np.concatenate([J * Nb + rows for J in range(n)])
    scale = np.abs(ra).max(axis=0)
    scale[1:4] = scale[1:4].max()
    assert (np.abs(rb[rows_all] - ra) / scale).max() < 1e-9


def test_phase_lag_needs_hb_and_cyclic(oracle_binding):
    w = cases.annular_sector(3, 4, 4, ordering_mode="natural")
    h = abi.CaseHandle(oracle_binding, w.mesh, cases.make_config(oracle_binding, w.settings))
    mode = np.zeros(len(w.mesh.patches), np.int32)
    with pytest.raises(abi.IcsError):
        h.set_phase_lag((mode, np.zeros((len(mode), 1, 1))))
