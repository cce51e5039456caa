"""Generate the golden vectors in this directory from the oracle.

The reference ships no golden data, so these fixtures record the oracle's
outputs (after the oracle passed the analytic known-answer tests in
tests/test_oracle.py) on small seeded workloads: the face fluxes, the matrix
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

CASES = {
    "tube_ausm_first_order": (lambda: cases.shock_tube(64), {}),
    "bump_hllc_muscl_venkat": (lambda: cases.bump_channel(12, 5, 3, ordering_mode="colour", flux="HLLC"), {}),
    "bump_roe_vanleer": (lambda: cases.bump_channel(10, 4, 3, ordering_mode="natural", flux="ROE"),
                         dict(recon_rho=1, recon_U=1, recon_T=1)),
    "box_ausm_muscl_minmod": (lambda: cases.random_box(5), dict(recon_rho=4, recon_U=4, recon_T=4)),
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
    h.set_primitive(w.p, w.U, w.T)
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
