"""Independent cases stacked in one handle (ics_set_cases) on the GPU.

A stack runs every kernel of a pseudo iteration once for all its cases while
each case keeps its own GMRES scalars, stop test, SER pseudo Courant number and
pseudotimeControl.  Checked here:
  * a case's trajectory in the stack follows a handle of its own (FP64, 1e-10
    of each field's max-norm after the dual-time steps of the shock tubes and
    the steady iterations of the bump channels), with the same number of
    pseudo iterations per time step and the same rho L2 residuals, and follows
    the oracle run of that case alone (1e-9);
  * a case's results do not depend on the other cases in the stack: the same
    case in two different stacks (other cases, other order) is bit-identical,
    in FP64 and in mixed precision;
  * invalid stacks are refused.
"""

import numpy as np
import pytest

from icsfoam_gb300 import abi, cases

from test_gpu_parity import perturb, relerr  # noqa: E402

pytestmark = pytest.mark.gpu

# 64 .. 2600 cells: one to three reduction segments per case
TUBES = (300, 1500, 64, 2600, 700)


def _tubes(sizes):
    return [cases.shock_tube(n, ordering_mode="colour") for n in sizes]


def _bumps():
    # perturbed states (as the parity tests use): from the uniform start the
    # y and z momentum residuals are round-off, and the GMRES stop test's
    # relative criterion divides them by round-off initial residuals, so a
    # different summation order changes the number of restart cycles
    return [perturb(cases.bump_channel(8, 4, 2, ordering_mode="colour"), seed=1),
            perturb(cases.bump_channel(12, 6, 3, ordering_mode="colour"), seed=2),
            perturb(cases.bump_channel(10, 4, 2, ordering_mode="colour"), seed=3)]


def _open(b, w, precision=0):
    h = abi.CaseHandle(b, w.mesh, cases.make_config(b, w.settings, precision=precision))
    return h


def run_stack(b, ws, steps, precision=0, pseudo=None):
    """Time steps of the stacked cases (pseudo: fixed pseudo iterations per
    call for a steady case); returns per-case states, pseudo iterations per
    case and step, and per-case rho L2 histories."""
    w, start = cases.stack_cases(ws)
    h = _open(b, w, precision)
    h.set_cases(start)
    h.set_primitive(w.p, w.U, w.T)
    n = len(ws)
    its = np.zeros((steps, n), int)
    l2 = [[] for _ in range(n)]
    for s in range(steps):
        if pseudo is None:
            h.begin_time_step()
        k = 0
        while h.pseudo_loop() if pseudo is None else k < pseudo:
            live = ~h.case_stats()["frozen"]
            h.pseudo_iteration()
            its[s] += live
            st = h.case_stats()["rho_l2"]
            for c in np.nonzero(live)[0]:
                l2[c].append(st[c])
            k += 1
    W = h.get_state()["W"]
    return [W[start[c]:start[c + 1]].copy() for c in range(n)], its, l2


def run_single(b, w, steps, precision=0, pseudo=None):
    h = _open(b, w, precision)
    h.set_primitive(w.p, w.U, w.T)
    its = np.zeros(steps, int)
    l2 = []
    for s in range(steps):
        if pseudo is None:
            h.begin_time_step()
        k = 0
        while h.pseudo_loop() if pseudo is None else k < pseudo:
            st = h.pseudo_iteration()
            its[s] += 1
            l2.append(st.rho_l2_residual)
            k += 1
    return h.get_state()["W"], its, l2


def rel(a, b):
    """Max error per equation relative to that equation's max-norm (the
    momentum components share one scale), as the parity tests measure."""
    return relerr(a, b)


@pytest.mark.parametrize("kind", ["tubes", "bumps"])
def test_stacked_cases_follow_their_own_handles(gpu_binding, kind):
    ws, steps, pseudo = (_tubes(TUBES), 3, None) if kind == "tubes" else (_bumps(), 1, 12)
    Ws, its, l2 = run_stack(gpu_binding, ws, steps, pseudo=pseudo)
    for c, w in enumerate(ws):
        W1, its1, l21 = run_single(gpu_binding, w, steps, pseudo=pseudo)
        assert np.array_equal(its[:, c], its1), (c, its[:, c], its1)
        assert rel(Ws[c], W1) < 1e-10, (c, rel(Ws[c], W1))
        assert np.allclose(l2[c], l21, rtol=1e-9, atol=0), c


def test_stacked_tubes_follow_the_oracle(gpu_binding, oracle_binding):
    ws = _tubes((120, 400, 64))
    Ws, its, _ = run_stack(gpu_binding, ws, 2)
    for c, w in enumerate(ws):
        Wo, itso, _ = run_single(oracle_binding, w, 2)
        assert np.array_equal(its[:, c], itso)
        assert rel(Ws[c], Wo) < 1e-9, (c, rel(Ws[c], Wo))


@pytest.mark.parametrize("precision", [0, 1])
def test_a_case_does_not_depend_on_the_stack(gpu_binding, precision):
    a = _tubes(TUBES)
    b = _tubes((1800,) + TUBES[::-1])  # another case in front, the order reversed
    Wa, itsa, _ = run_stack(gpu_binding, a, 2, precision)
    Wb, itsb, _ = run_stack(gpu_binding, b, 2, precision)
    for c in range(len(TUBES)):
        cb = len(TUBES) - c  # position of case c in stack b
        assert np.array_equal(itsa[:, c], itsb[:, cb])
        assert np.array_equal(Wa[c], Wb[cb]), (precision, c)


def test_invalid_stacks_are_refused(gpu_binding):
    w, start = cases.stack_cases(_tubes((40, 60)))
    h = _open(gpu_binding, w)
    for bad in ([0, 40], [0, 60, 40, 100], [0, 0, 100], [1, 40, 100]):
        with pytest.raises(abi.IcsError):
            h.set_cases(np.array(bad))
    # a face joining two cases: split one tube in the middle
    wt = cases.shock_tube(50, ordering_mode="natural")
    ht = _open(gpu_binding, wt)
    with pytest.raises(abi.IcsError):
        ht.set_cases(np.array([0, 25, 50]))
    h.set_cases(start)
    with pytest.raises(abi.IcsError):
        h.scalar_enable(np.full(w.mesh.n_cells, 0.1), D=0.0, recon=0)
    with pytest.raises(abi.IcsError):
        h.save_checkpoint()
    plain = _open(gpu_binding, cases.shock_tube(100, ordering_mode="colour"))
    plain.set_primitive(*(np.ones(100) * 1e5, np.zeros((100, 3)), np.ones(100) * 300.0))
    blob = plain.save_checkpoint()
    w2, start2 = cases.stack_cases(_tubes((40, 60)))
    h2 = _open(gpu_binding, w2)
    h2.set_cases(start2)
    with pytest.raises(abi.IcsError):
        h2.load_checkpoint(blob)
