"""Host-side mirror of the reference's plugin interface for the hot path.

The reference selects its hot-path objects from OpenFOAM dictionaries
through runtime-selection tables:

* ``convectiveFluxScheme::New`` keyed by ``fvSchemes/convectiveFluxScheme/
  fluxScheme`` (newConvectiveFluxScheme.C:39-69) with the virtuals
  ``calcFlux(phi, phiUp, phiEp)`` and ``createConvectiveJacobian(coupledMatrix&,
  ddtCoeff)`` (convectiveFluxScheme.H:219-230);
* ``coupledMatrix::solver::New`` keyed by ``fvSolution/flowSolver/solver``
  (coupledMatrixSolver.C:41-67) with ``solveDelta`` (gmres.C:772-1107), its
  preconditioner keyed by ``preconditioner`` (coupledMatrix.H:296-369);
* ``pseudotimeControl`` reading ``fvSolution/pseudoTime``
  (pseudotimeControl.C:42-63).

Here the same dictionary keys and names select the GB300 path; ``GPU``
suffixed names (``AUSMPlusUpGPU``, ``HLLCGPU``, ``ROEGPU``, ``GMRESGPU``) are
accepted as aliases, which is how an OpenFOAM case switches to this path.
Unknown names raise ``ValueError`` where the reference raises FatalError.
Dictionaries are plain Python dicts of the OpenFOAM entries.
"""

from __future__ import annotations

from typing import Dict, Optional

import numpy as np

from . import abi, gpu
from . import mesh as _mesh

_FLUX = {"AUSMPlusUp": abi.FLUX["AUSMPlusUp"], "HLLC": abi.FLUX["HLLC"], "ROE": abi.FLUX["ROE"]}
_DDT = {"steadyState": 0, "Euler": 1, "backward": 2}


def _strip_gpu(name: str) -> str:
    return name[:-3] if name.endswith("GPU") else name


def _switch(v) -> int:
    if isinstance(v, str):
        return int(v.lower() in ("true", "on", "yes", "1"))
    return int(bool(v))


def reconstruction_scheme(entry: str, grad_entry: Optional[str]) -> int:
    """Map an ``interpolationSchemes`` entry (plus its gradient scheme) to ICS_RECON_*."""
    words = entry.split()
    if not words:
        raise ValueError("empty interpolation scheme")
    kind = words[0]
    if kind == "upwind":
        return abi.RECON["upwind"]
    if kind == "vanLeer":
        return abi.RECON["vanLeer"]
    if kind in ("Minmod", "minmod"):
        return abi.RECON["Minmod"]
    if kind == "linearUpwind":
        g = (grad_entry or "").split()
        if g and g[0] == "cellLimited<Venkatakrishnan>":
            return abi.RECON["MUSCLVenkatakrishnan"]
        if g and g[0] in ("cellLimited", "cellLimited<minmod>"):
            return abi.RECON["MUSCLMinmod"]
        raise ValueError("linearUpwind needs a cellLimited gradient scheme, got %r" % grad_entry)
    raise ValueError("Unknown interpolation scheme %r" % kind)


def cell_limited_coeff(grad_entry: Optional[str]) -> float:
    """The coefficient k of ``cellLimited<limiter> Gauss linear k`` (OpenFOAM
    cellLimitedGrad: k in [0, 1]; 1 when omitted).  k = 0 (no limiting) is
    not provided."""
    words = (grad_entry or "").split()
    if len(words) >= 4 and words[1] == "Gauss":
        k = float(words[3])
    elif len(words) >= 2 and words[1] != "Gauss":
        k = float(words[-1])
    else:
        k = 1.0
    if not 0.0 < k <= 1.0:
        raise ValueError("cellLimited coefficient must be in (0, 1], got %g" % k)
    return k


def config_from_dicts(binding: abi.Binding, fvSchemes: Dict, fvSolution: Dict, thermo: Optional[Dict] = None):
    """Build an ics_config from fvSchemes / fvSolution / thermophysical entries."""
    cfg = binding.default_config()
    cfs = fvSchemes.get("convectiveFluxScheme", {})
    name = _strip_gpu(cfs.get("fluxScheme", "AUSMPlusUp"))
    if name not in _FLUX:
        raise ValueError("Unknown convectiveFluxScheme type %s; valid types: %s" % (name, sorted(_FLUX)))
    cfg.flux_scheme = _FLUX[name]
    cfg.low_mach_ausm = _switch(cfs.get("lowMachAusm", True))
    cfg.entropy_fix_coeff = float(cfs.get("entropyFixCoeff", 0.05))
    # viscousFluxScheme { LaxFriedrichJacobian true; } (viscousFluxScheme.C:107)
    cfg.viscous_lf_jacobian = _switch(fvSchemes.get("viscousFluxScheme", {}).get("LaxFriedrichJacobian", True))
    ddt = fvSchemes.get("ddtSchemes", {}).get("default", "dualTime rPseudoDeltaT steadyState").split()
    if len(ddt) < 3 or ddt[0] != "dualTime" or ddt[-1] not in _DDT:
        raise ValueError("ddtSchemes default must be 'dualTime rPseudoDeltaT <steadyState|Euler|backward>'")
    cfg.ddt_scheme = _DDT[ddt[-1]]
    interp = fvSchemes.get("interpolationSchemes", {})
    grads = fvSchemes.get("gradSchemes", {})
    coeffs = set()
    for field, attr in (("rho", "recon_rho"), ("U", "recon_U"), ("T", "recon_T")):
        entry = interp.get("reconstruct(%s)" % field, "upwind")
        gname = entry.split()[1] if len(entry.split()) > 1 else None
        gentry = grads.get(gname, grads.get("default")) if gname else None
        setattr(cfg, attr, reconstruction_scheme(entry, gentry))
        if entry.split()[0] == "linearUpwind":
            coeffs.add(cell_limited_coeff(gentry))
    if len(coeffs) > 1:
        raise ValueError("different cellLimited coefficients per reconstructed field are not provided: %s"
                         % sorted(coeffs))
    cfg.limiter_coeff = coeffs.pop() if coeffs else 1.0
    fs = fvSolution.get("flowSolver", {})
    sname = _strip_gpu(fs.get("solver", "GMRES"))
    if sname not in abi.SOLVER:
        raise ValueError("Unknown solver type %s; valid types: %s" % (sname, sorted(abi.SOLVER)))
    cfg.solver = abi.SOLVER[sname]
    sd = fs.get(sname, fs.get(sname + "GPU", {}))
    if sname == "smoothSolverCoupled":
        if sd.get("smoother", "Jacobi") != "Jacobi":
            raise ValueError("Unknown smoother %s; valid types: [Jacobi]" % sd.get("smoother"))
        cfg.n_sweeps = int(sd.get("nSweeps", 1))
    else:
        pc = sd.get("preconditioner", "LUSGS")
        if pc not in abi.PRECON:
            raise ValueError("Unknown preconditioner %s" % pc)
        cfg.preconditioner = abi.PRECON[pc]
        cfg.n_directions = int(sd["nDirections"])
    cfg.max_iter = int(sd.get("maxIter", 1000))
    cfg.min_iter = int(sd.get("minIter", 0))
    cfg.tolerance = float(sd["tolerance"])
    cfg.rel_tol = float(sd["relTol"])
    prec = fs.get("precision", sd.get("precision", "fp64"))
    if prec not in abi.PRECISION:
        raise ValueError("precision must be fp64 or mixed")
    cfg.precision = abi.PRECISION[prec]
    pt = fvSolution.get("pseudoTime", {})
    cfg.n_pseudo_corr = int(pt.get("nPseudoCorr", 20))
    cfg.n_pseudo_corr_min = int(pt.get("nPseudoCorrMin", 1))
    cfg.pseudo_tol = float(pt["pseudoTol"])
    cfg.pseudo_tol_rel = float(pt["pseudoTolRel"])
    cfg.pseudo_co_num = float(pt.get("pseudoCoNum", 1))
    cfg.pseudo_co_num_min = float(pt.get("pseudoCoNumMin", 0.1))
    cfg.pseudo_co_num_max = float(pt.get("pseudoCoNumMax", 25))
    cfg.pseudo_co_max_increase = float(pt.get("pseudoCoNumMaxIncreaseFactor", 1.25))
    cfg.pseudo_co_min_decrease = float(pt.get("pseudoCoNumMinDecreaseFactor", 0.1))
    cfg.local_timestepping = _switch(pt.get("localTimestepping", True))
    cfg.local_timestepping_bounding = _switch(pt.get("localTimesteppingBounding", True))
    lb = float(pt.get("localTimesteppingLowerBound", 0.95))
    cfg.local_timestepping_lower_bound = min(max(lb, 0.0), 0.99)
    cfg.reset_pseudo = _switch(pt.get("resetPseudo", False))
    cfg.rho_min = float(pt.get("rhoMin", -1e15))
    cfg.T_min = float(pt.get("TMin", 1e-15))
    cfg.T_max = float(pt.get("TMax", 1e15))
    if thermo:
        if "R" in thermo:
            cfg.R = float(thermo["R"])
        if "Cp" in thermo:
            cfg.Cp = float(thermo["Cp"])
    return cfg


class Case:
    """A case resident on the GPU: mesh, fields and the selected hot-path objects."""

    def __init__(self, mesh: _mesh.Mesh, fvSchemes: Dict, fvSolution: Dict, thermo: Optional[Dict] = None,
                 binding: Optional[abi.Binding] = None):
        self.binding = binding or gpu.binding()
        self.cfg = config_from_dicts(self.binding, fvSchemes, fvSolution, thermo)
        self.handle = abi.CaseHandle(self.binding, mesh, self.cfg)
        self.mesh = mesh
        self.flux = convectiveFluxScheme(self)
        self.control = pseudotimeControl(self)

    def setFields(self, p, U, T):
        self.handle.set_primitive(p, U, T)


class convectiveFluxScheme:
    """calcFlux / createConvectiveJacobian of the selected scheme."""

    def __init__(self, case: Case):
        self.case = case

    def calcFlux(self):
        """Returns (phi, phiUp, phiEp) over internal then boundary faces."""
        return self.case.handle.calc_flux()

    def residual(self):
        """residualsUpdate.H + setCoAndDeltaT.H: matrix source R*V [N][5]."""
        return self.case.handle.residual()

    def createConvectiveJacobian(self):
        self.case.handle.assemble_jacobian()
        return coupledMatrix(self.case)


class coupledMatrix:
    """The assembled 5x5 block system of one pseudo iteration."""

    def __init__(self, case: Case):
        self.case = case

    def matrixMul(self, x: np.ndarray) -> np.ndarray:
        return self.case.handle.matrix_mul(x)

    def blocks(self):
        """(diag [N,5,5], lower [F,5,5], upper [F,5,5]) in LDU form."""
        return self.case.handle.get_jacobian()

    def precondition(self, r: np.ndarray) -> np.ndarray:
        return self.case.handle.precondition(r)

    def solveForIncr(self):
        perf, dW, status = self.case.handle.solve_increment(allow=(abi.ICS_OK, abi.ICS_ERR_BREAKDOWN))
        return perf, dW


class pseudotimeControl:
    """pseudotimeControl::loop over the handle's pseudo iterations."""

    def __init__(self, case: Case):
        self.case = case

    def loop(self) -> bool:
        return self.case.handle.pseudo_loop()

    def iterate(self):
        return self.case.handle.pseudo_iteration()
