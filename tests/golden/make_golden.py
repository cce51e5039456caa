"""Generate the golden vectors in this directory from the oracle.

The reference ships no golden data, so these fixtures record the oracle's
outputs (after the oracle passed the analytic known-answer tests in
tests/test_oracle.py, test_cyclic.py and test_phase_lag.py) on small seeded
workloads -- plain, rotating-zone, cyclic and phase-lag cases: the face fluxes, the matrix
source R*V, the Jacobian action on a fixed vector, one GMRES increment and a
three-iteration residual history.  Both the oracle (CPU tests) and the CUDA
path (GPU tests) are checked against them.

    python tests/golden/make_golden.py
"""

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from icsfoam_gb300 import abi, cases  # noqa: E402

def _hb_sector():
    from icsfoam_gb300 import hb as HB

    base = cases.annular_sector(4, 6, 5, ordering_mode="colour", flux="AUSMPlusUp")
    n = 3
    om = HB.omega_list([50.0], [1])
    t = HB.select_instants(om, n, None)
    st = HB.stack_instances(base.mesh, n)
    rep = lambda a: np.concatenate([a] * n)
    w = cases.Workload("hb_sector", st, rep(base.p), rep(base.U), rep(base.T), dict(base.settings),
                       hb=(n, HB.hb_operator(om, t)))
    w.plag = HB.phase_lag_setup(st, n, om, t, 0.7, cyl_coords=True)
    return w


def _periodic_bump():
    from icsfoam_gb300 import mesh as M

    g = cases.bump_points(8, 4, 3, width=0.3)
    inlet = M.Patch("inlet", M.PATCH_TOTAL_INLET, p0=1.0e5, T0=300.0)
    outlet = M.Patch("outlet", M.PATCH_PRESSURE_OUTLET, p=0.75e5)
    wall = M.Patch("walls", M.PATCH_SLIP, is_wall=True)
    a, b = M.cyclic_pair("front", "back", separation=(0.0, 0.0, -0.3))
    m = M.hex_mesh(g, {"xmin": inlet, "xmax": outlet, "ymin": wall, "ymax": wall, "zmin": a, "zmax": b})
    N = m.n_cells
    w = cases.bump_channel(8, 4, 3)
    return cases.Workload("bump_periodic", m, np.full(N, w.p[0]), np.tile(w.U[:1], (N, 1)), np.full(N, w.T[0]),
                          dict(w.settings))


def _setup(h, w):
    """Zone / coupling set-up after the initial state (MRF zones, phase lag)."""
    from icsfoam_gb300 import mrf as MRF

    if getattr(w, "mrf", None):
        h.set_mrf(MRF.frame_fields(w.mesh, *w.mrf))
    if getattr(w, "plag", None) is not None:
        h.set_phase_lag(w.plag)


# name: (workload, ics_config overrides)
CASES = {
    "tube_ausm_first_order": (lambda: cases.shock_tube(64), {}),
    "bump_hllc_muscl_venkat": (lambda: cases.bump_channel(12, 5, 3, ordering_mode="colour", flux="HLLC"), {}),
    "bump_roe_vanleer": (lambda: cases.bump_channel(10, 4, 3, ordering_mode="natural", flux="ROE"),
                         dict(recon_rho=1, recon_U=1, recon_T=1)),
    "box_ausm_muscl_minmod": (lambda: cases.random_box(5), dict(recon_rho=4, recon_U=4, recon_T=4)),
    # rotational cyclic sector with its rotating zone (MRF)
    "annulus_cyclic_mrf_hllc": (lambda: cases.annular_sector(5, 6, 6, ordering_mode="colour", flux="HLLC"), {}),
    # translational cyclic (periodic span)
    "bump_periodic_roe": (_periodic_bump, dict(flux_scheme=2)),
    # Harmonic Balance instances with phase-lag cyclic sides
    "hb_sector_phase_lag_ausm": (_hb_sector, {}),
}


def perturb(w, seed=11, amp=0.02):
    rng = np.random.default_rng(seed)
    N = w.mesh.n_cells
    w.p = w.p * (1 + amp * rng.uniform(-1, 1, N))
    w.T = w.T * (1 + amp * rng.uniform(-1, 1, N))
    w.U = w.U + 2.0 * rng.uniform(-1, 1, (N, 3)) * (np.array(w.mesh.solution_d) > 0)
    return w


def compute(binding, name):
    build, over = CASES[name]
    w = perturb(build())
    cfg = cases.make_config(binding, w.settings, **over)
    h = abi.CaseHandle(binding, w.mesh, cfg)
    if w.hb:
        h.set_hb(*w.hb)
    h.set_primitive(w.p, w.U, w.T)
    _setup(h, w)
    if w.settings.get("ddt_scheme", 0):
        h.begin_time_step()
    phi, phiU, phiE = h.calc_flux()
    src = h.residual()
    h.assemble_jacobian()
    x = np.random.default_rng(5).standard_normal((w.mesh.n_cells, 5))
    Ax = h.matrix_mul(x)
    perf, dW, _ = h.solve_increment()
    h.update_fields()
    hist = []
    for _ in range(3):
        s = h.pseudo_iteration()
        hist.append(s.rho_l2_residual)
    return dict(phi=phi, phiU=phiU, phiE=phiE, src=src, x=x, Ax=Ax, dW=dW, hist=np.array(hist),
                W=h.get_state()["W"], gmres_cycles=np.array(perf.n_iterations))


def main():
    import oracle

    b = oracle.binding()
    for name in CASES:
        d = compute(b, name)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **d)
        print(name, {k: v.shape for k, v in d.items()})


if __name__ == "__main__":
    main()
