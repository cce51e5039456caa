"""GPU path vs the oracle at the full sizes of the workloads.

The other parity tests run on meshes of a few thousand cells; these repeat
the core comparisons on the meshes the throughput figures are measured on,
from a perturbed state (2% random perturbation of p, T and U, so every cell
carries a non-trivial residual):

* bump channel 256x64x64 (1,048,576 cells; HLLC + MUSCL/Venkatakrishnan,
  colour-blocked numbering): residual source, Jacobian action, LU-SGS
  application, then two full pseudo iterations in lockstep with the
  residual vector of every iteration compared;
* randomised viscous box 200^3 (8,000,000 cells; AUSM+up + MUSCL, Sutherland
  viscosity, RCM numbering, so the many-level LU-SGS sweeps);
* Harmonic Balance on the rotational-cyclic annular sector 32x64x128 with one
  harmonic (3 instances of 262,144 cells, spectral source and couplings);
* swept bump 240x128x128 (3,932,160 cells; HLLC + MUSCL).

Tolerances: 1e-12 of each equation's max-norm for the residual source, the
Jacobian action and the preconditioner (as in the small-mesh tests).  Over a
pseudo iteration the GMRES increment carries the Krylov solver's round-off;
the state and the next residual are compared at 1e-10.

The oracle is sequential: each evaluation takes seconds to a minute at these
sizes, so every test makes only the comparisons listed.
"""

import numpy as np
import pytest

from icsfoam_gb300 import abi, cases

from test_gpu_parity import perturb, relerr  # noqa: E402

pytestmark = pytest.mark.gpu

FULL = {
    "bump_256x64x64": lambda: cases.bump_channel(256, 64, 64, ordering_mode="colour"),
    "random_box_200": lambda: cases.random_box(200),
    "hb3_annulus_32x64x128": lambda: cases.hb_annular_sector(32, 64, 128, harmonics=1),
    "swept_bump_240x128x128": lambda: cases.swept_bump(240, 128, 128),
}


def _open(binding, w):
    h = abi.CaseHandle(binding, w.mesh, cases.make_config(binding, w.settings))
    if w.hb:
        h.set_hb(*w.hb)
    h.set_primitive(w.p, w.U, w.T)
    return h


def _report(name, **errs):
    print("\n[fullsize] %s %s" % (name, " ".join("%s=%.3e" % kv for kv in errs.items())))


@pytest.mark.parametrize("name", list(FULL))
def test_fullsize_residual_jacobian_preconditioner(oracle_binding, gpu_binding, name):
    w = perturb(FULL[name]())
    ho, hg = _open(oracle_binding, w), _open(gpu_binding, w)
    so, sg = ho.residual(), hg.residual()
    e_res = relerr(sg, so)
    for h in (ho, hg):
        h.assemble_jacobian()
    x = np.random.default_rng(11).standard_normal((w.mesh.n_cells, 5))
    e_mv = relerr(hg.matrix_mul(x), ho.matrix_mul(x))
    e_pc = relerr(hg.precondition(x), ho.precondition(x))
    _report(name, residual=e_res, matrix_mul=e_mv, precondition=e_pc)
    assert e_res < 1e-12
    assert e_mv < 1e-12
    assert e_pc < 1e-12


def test_fullsize_bump_two_pseudo_iterations(oracle_binding, gpu_binding):
    """Two pseudo iterations of the 1,048,576-cell bump channel in lockstep:
    the residual source at the start of each iteration, the GMRES cycle
    counts and initial residuals, the updated state and boundary values."""
    w = perturb(FULL["bump_256x64x64"]())
    ho, hg = _open(oracle_binding, w), _open(gpu_binding, w)
    errs = {}
    for it in range(2):
        so, sg = ho.residual(), hg.residual()
        errs["residual_%d" % it] = relerr(sg, so)
        for h in (ho, hg):
            h.assemble_jacobian()
        po, dWo, _ = ho.solve_increment()
        pg, dWg, _ = hg.solve_increment()
        assert pg.n_iterations == po.n_iterations, it
        errs["init_res_%d" % it] = float(np.max(np.abs(np.array(pg.init_res) - np.array(po.init_res)) /
                                                np.abs(np.array(po.init_res))))
        errs["increment_%d" % it] = relerr(dWg, dWo)
        ho.update_fields()
        hg.update_fields()
        errs["state_%d" % it] = relerr(hg.get_state()["W"], ho.get_state()["W"])
    errs["residual_2"] = relerr(hg.residual(), ho.residual())
    _report("bump_256x64x64 lockstep", **errs)
    assert errs["residual_0"] < 1e-12
    for it in range(2):
        assert errs["init_res_%d" % it] < 1e-11
        assert errs["increment_%d" % it] < 1e-10
        assert errs["state_%d" % it] < 1e-10
    assert errs["residual_1"] < 1e-10
    assert errs["residual_2"] < 1e-10
