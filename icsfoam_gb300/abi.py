"""ctypes mirror of include/icsfoam_gb300.h.

``Binding`` wraps one shared library that exports the C ABI under a given
symbol prefix ("ics_" for the CUDA library).  ``CaseHandle`` owns one
``ics_handle`` plus the numpy arrays whose pointers were handed over.
"""

from __future__ import annotations

import ctypes as C
from typing import Optional

import numpy as np

from . import mesh as _mesh

ICS_OK = 0
ICS_ERR_ARG = 1
ICS_ERR_CUDA = 2
ICS_ERR_NONFINITE = 3
ICS_ERR_BREAKDOWN = 4
ICS_ERR_DIAG = 5
ICS_ERR_SCHEME = 6
ICS_ERR_STATE = 7
ICS_ERR_NOMEM = 8
ICS_ERR_TIMEOUT = 9

STATUS_NAMES = {
    0: "ok", 1: "invalid argument", 2: "CUDA error", 3: "non-finite value",
    4: "Krylov breakdown", 5: "zero diagonal", 6: "unknown scheme",
    7: "call order", 8: "out of device memory", 9: "device wait timeout",
}

FLUX = {"AUSMPlusUp": 0, "HLLC": 1, "ROE": 2}
RECON = {"upwind": 0, "vanLeer": 1, "Minmod": 2, "MUSCLVenkatakrishnan": 3, "MUSCLMinmod": 4}
DDT = {"steadyState": 0, "Euler": 1, "backward": 2}
PRECON = {"none": 0, "LUSGS": 1, "Jacobi": 2}
SOLVER = {"GMRES": 0, "smoothSolverCoupled": 1}
PRECISION = {"fp64": 0, "mixed": 1}


class IcsError(RuntimeError):
    def __init__(self, status: int, where: str, msg: str = ""):
        super().__init__(f"{where}: {STATUS_NAMES.get(status, status)} ({status}) {msg}".strip())
        self.status = status


class PatchDesc(C.Structure):
    _fields_ = [("kind", C.c_int32), ("is_wall", C.c_int32), ("p", C.c_double), ("T", C.c_double),
                ("U", C.c_double * 3), ("p0", C.c_double), ("T0", C.c_double), ("rotation", C.c_double * 9)]


class MeshDesc(C.Structure):
    _fields_ = [
        ("n_cells", C.c_int32), ("n_faces", C.c_int32), ("n_bfaces", C.c_int32), ("n_patches", C.c_int32),
        ("owner", C.c_void_p), ("neighbour", C.c_void_p),
        ("Sf", C.c_void_p), ("Cf", C.c_void_p), ("weights", C.c_void_p),
        ("delta_coeffs", C.c_void_p), ("nonorth_delta_coeffs", C.c_void_p),
        ("C", C.c_void_p), ("V", C.c_void_p),
        ("b_cell", C.c_void_p), ("b_patch", C.c_void_p), ("b_Sf", C.c_void_p), ("b_Cf", C.c_void_p),
        ("b_delta_coeffs", C.c_void_p), ("patches", C.POINTER(PatchDesc)),
        ("solution_d", C.c_int32 * 3),
        ("b_partner", C.c_void_p), ("b_weights", C.c_void_p), ("b_nbr_d", C.c_void_p),
        ("b_nonorth_delta_coeffs", C.c_void_p),
    ]


class Config(C.Structure):
    _fields_ = [
        ("R", C.c_double), ("Cp", C.c_double),
        ("mu", C.c_double), ("Pr", C.c_double), ("As", C.c_double), ("Ts", C.c_double),
        ("sutherland", C.c_int32), ("viscous", C.c_int32),
        ("flux_scheme", C.c_int32), ("low_mach_ausm", C.c_int32), ("entropy_fix_coeff", C.c_double),
        ("recon_rho", C.c_int32), ("recon_U", C.c_int32), ("recon_T", C.c_int32),
        ("ddt_scheme", C.c_int32), ("delta_t", C.c_double),
        ("solver", C.c_int32), ("preconditioner", C.c_int32), ("n_directions", C.c_int32),
        ("max_iter", C.c_int32), ("min_iter", C.c_int32),
        ("tolerance", C.c_double), ("rel_tol", C.c_double),
        ("precision", C.c_int32),
        ("n_pseudo_corr", C.c_int32), ("n_pseudo_corr_min", C.c_int32),
        ("pseudo_tol", C.c_double), ("pseudo_tol_rel", C.c_double),
        ("pseudo_co_num", C.c_double), ("pseudo_co_num_min", C.c_double), ("pseudo_co_num_max", C.c_double),
        ("pseudo_co_max_increase", C.c_double), ("pseudo_co_min_decrease", C.c_double),
        ("local_timestepping", C.c_int32), ("local_timestepping_bounding", C.c_int32),
        ("local_timestepping_lower_bound", C.c_double),
        ("reset_pseudo", C.c_int32),
        ("rho_min", C.c_double), ("T_min", C.c_double), ("T_max", C.c_double),
        ("n_sweeps", C.c_int32),
        ("viscous_lf_jacobian", C.c_int32),
        ("limiter_coeff", C.c_double),
    ]


class SolverPerf(C.Structure):
    _fields_ = [("init_res", C.c_double * 5), ("final_res", C.c_double * 5),
                ("n_iterations", C.c_int32), ("converged", C.c_int32)]

    def as_dict(self):
        return {"init_res": list(self.init_res), "final_res": list(self.final_res),
                "n_iterations": int(self.n_iterations), "converged": bool(self.converged)}


class IterStats(C.Structure):
    _fields_ = [("perf", SolverPerf), ("rho_l2_residual", C.c_double), ("pseudo_co_mean", C.c_double),
                ("bounded_cells", C.c_int32), ("status", C.c_int32)]


class Tuning(C.Structure):
    _fields_ = [("face_block", C.c_int32), ("grad_block", C.c_int32), ("mgs_blocks", C.c_int32),
                ("fused_operator", C.c_int32), ("from_cache", C.c_int32), ("reverse_rows", C.c_int32)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class KrylovOpts(C.Structure):
    _fields_ = [("n_directions", C.c_int32), ("max_cycles", C.c_int32), ("rel_tol", C.c_double),
                ("precision", C.c_int32), ("preconditioner", C.c_int32), ("pseudo_time", C.c_int32)]


class KrylovResult(C.Structure):
    _fields_ = [("iterations", C.c_int32), ("cycles", C.c_int32), ("rel_residual", C.c_double),
                ("converged", C.c_int32)]


# exported functions: name -> (restype, argtypes)
_P = C.c_void_p
_FUNCS = {
    "default_config": (None, [C.POINTER(Config)]),
    "create": (C.c_int, [C.POINTER(MeshDesc), C.POINTER(Config), C.POINTER(_P)]),
    "destroy": (C.c_int, [_P]),
    "set_config": (C.c_int, [_P, C.POINTER(Config)]),
    "last_error": (C.c_int, [_P, C.c_char_p, C.c_int32]),
    "set_primitive": (C.c_int, [_P, _P, _P, _P]),
    "set_boundary_state": (C.c_int, [_P, _P, _P, _P, _P]),
    "get_boundary_state": (C.c_int, [_P, _P, _P, _P, _P]),
    "get_state": (C.c_int, [_P, _P, _P, _P, _P]),
    "set_conservative": (C.c_int, [_P, _P, C.c_int32]),
    "set_pseudo_co": (C.c_int, [_P, _P]),
    "get_pseudo_co": (C.c_int, [_P, _P, _P]),
    "calc_flux": (C.c_int, [_P, _P, _P, _P]),
    "residual": (C.c_int, [_P, _P]),
    "assemble_jacobian": (C.c_int, [_P]),
    "get_jacobian": (C.c_int, [_P, _P, _P, _P]),
    "matrix_mul": (C.c_int, [_P, _P, _P]),
    "precondition": (C.c_int, [_P, _P]),
    "solve_increment": (C.c_int, [_P, C.POINTER(SolverPerf), _P]),
    "update_fields": (C.c_int, [_P, C.POINTER(IterStats)]),
    "pseudo_iteration": (C.c_int, [_P, C.POINTER(IterStats)]),
    "begin_time_step": (C.c_int, [_P]),
    "pseudo_loop": (C.c_int, [_P, C.POINTER(C.c_int32)]),
    "set_hb": (C.c_int, [_P, C.c_int32, _P]),
    "set_hb_zone": (C.c_int, [_P, _P, C.c_int32, _P, _P]),
    "set_mrf": (C.c_int, [_P, _P, _P, _P, _P, C.c_int32]),
    "set_phase_lag": (C.c_int, [_P, _P, _P]),
    "scalar_enable": (C.c_int, [_P, _P, _P, _P, C.c_double, C.c_int32]),
    "scalar_transport": (C.c_int, [_P, C.c_int32, C.POINTER(SolverPerf)]),
    "get_scalar": (C.c_int, [_P, _P, _P]),
}

# measurement entry points (CUDA library only)
_MEASURE = {
    "profile": (C.c_int, [_P, C.c_int32]),
    "profile_read": (C.c_int, [_P, C.c_int32, C.POINTER(C.c_double), C.POINTER(C.c_int64)]),
    "launch_count": (C.c_int, [_P, C.POINTER(C.c_int64)]),
    "timer_start": (C.c_int, [_P]),
    "timer_stop": (C.c_int, [_P, C.POINTER(C.c_double)]),
    "measure_fp64_rate": (C.c_int, [_P, C.POINTER(C.c_double)]),
    "autotune": (C.c_int, [_P, C.POINTER(Tuning)]),
    "set_tuning": (C.c_int, [_P, C.POINTER(Tuning)]),
}

# allocation-free linear residual (CUDA library only; arguments are device pointers)
_MEASURE["linear_residual_noalloc"] = (C.c_int, [_P, _P, _P, _P])

# independent cases iterated concurrently (CUDA library only)
_MEASURE["pseudo_iteration_batch"] = (C.c_int, [_P, C.c_int32, _P, _P])

# independent cases stacked in one handle (CUDA library only)
_MEASURE["set_cases"] = (C.c_int, [_P, C.c_int32, _P])
_MEASURE["case_stats"] = (C.c_int, [_P, _P, _P, _P])

# bounded-wait probe (CUDA library only)
_MEASURE["test_sweep_timeout"] = (C.c_int, [_P, C.c_int32, C.c_int32])

# checkpoint / resume (CUDA library only)
_MEASURE["checkpoint_size"] = (C.c_int, [_P, C.POINTER(C.c_int64)])
_MEASURE["save_checkpoint"] = (C.c_int, [_P, _P, C.c_int64])
_MEASURE["load_checkpoint"] = (C.c_int, [_P, _P, C.c_int64])

# differentiation of the residual (CUDA library only)
_MEASURE["jvp"] = (C.c_int, [_P, _P, _P, C.c_int32])
_MEASURE["vjp"] = (C.c_int, [_P, _P, _P, C.c_int32])
_MEASURE["vjp_recompute"] = (C.c_int, [_P, _P, _P, C.c_int32])
_MEASURE["adjoint_solve"] = (C.c_int, [_P, _P, _P, C.POINTER(KrylovOpts), C.POINTER(KrylovResult)])
_MEASURE["tangent_solve"] = (C.c_int, [_P, _P, _P, C.POINTER(KrylovOpts), C.POINTER(KrylovResult)])
_MEASURE["pressure_force"] = (C.c_int, [_P, C.c_int32, _P, C.POINTER(C.c_double), _P])
_MEASURE["assemble_exact_jacobian"] = (C.c_int, [_P, C.POINTER(C.c_int64), C.POINTER(C.c_int32)])
_MEASURE["get_exact_jacobian"] = (C.c_int, [_P, _P, _P, _P])

KERNEL_CLASSES = ("fields", "grad", "face", "bface", "cellres", "jac_boundary", "jac_rows", "jacobi_inv", "spmv",
                  "lusgs_fwd", "lusgs_rev", "jacobi", "mgs", "vector", "scalar", "update", "bc", "bound", "visc",
                  "tangent", "exact", "op0", "op1", "passive", "adjoint")

EXPORTED = tuple(_FUNCS) + tuple(_MEASURE)


class Binding:
    """Typed access to one library exporting the C ABI with ``prefix``."""

    def __init__(self, lib: C.CDLL, prefix: str):
        self.lib = lib
        self.prefix = prefix
        self.fn = {}
        for name, (res, args) in _FUNCS.items():
            f = getattr(lib, prefix + name)
            f.restype = res
            f.argtypes = args
            self.fn[name] = f
        for name, (res, args) in _MEASURE.items():
            f = getattr(lib, prefix + name, None)
            if f is not None:
                f.restype = res
                f.argtypes = args
                self.fn[name] = f

    def default_config(self) -> Config:
        cfg = Config()
        self.fn["default_config"](C.byref(cfg))
        return cfg


def _ptr(a: Optional[np.ndarray]):
    if a is None:
        return None
    return a.ctypes.data


def pseudo_iteration_batch(handles):
    """One pseudo iteration on each of several independent handles at once.

    Returns (stats list, status list); raises on the first failing handle.
    """
    if not handles:
        return [], []
    b = handles[0].b
    n = len(handles)
    arr = (C.c_void_p * n)(*[h.h.value for h in handles])
    stats = (IterStats * n)()
    status = (C.c_int32 * n)()
    st = b.fn["pseudo_iteration_batch"](arr, n, stats, status)
    if st != ICS_OK:
        bad = [k for k in range(n) if status[k] != ICS_OK]
        if not bad:  # rejected before any handle ran
            raise IcsError(st, b.prefix + "pseudo_iteration_batch")
        handles[bad[0]]._check(status[bad[0]], "pseudo_iteration_batch")
    return list(stats), list(status)


class CaseHandle:
    """One case (mesh + state) behind the C ABI of ``binding``."""

    def __init__(self, binding: Binding, mesh: _mesh.Mesh, cfg: Config):
        self.b = binding
        self.mesh = mesh
        self.N = mesh.n_cells
        self.F = mesh.n_faces
        self.B = mesh.n_bfaces
        self._keep = []
        desc = MeshDesc()
        desc.n_cells, desc.n_faces, desc.n_bfaces = self.N, self.F, self.B
        desc.n_patches = len(mesh.patches)

        def keep(a, dt):
            a = np.ascontiguousarray(a, dtype=dt)
            self._keep.append(a)
            return a.ctypes.data

        desc.owner = keep(mesh.owner, np.int32)
        desc.neighbour = keep(mesh.neighbour, np.int32)
        desc.Sf = keep(mesh.Sf, np.float64)
        desc.Cf = keep(mesh.Cf, np.float64)
        desc.weights = keep(mesh.weights, np.float64)
        desc.delta_coeffs = keep(mesh.delta_coeffs, np.float64)
        desc.nonorth_delta_coeffs = keep(mesh.nonorth_delta_coeffs, np.float64)
        desc.C = keep(mesh.C, np.float64)
        desc.V = keep(mesh.V, np.float64)
        desc.b_cell = keep(mesh.b_cell, np.int32)
        desc.b_patch = keep(mesh.b_patch, np.int32)
        desc.b_Sf = keep(mesh.b_Sf if self.B else np.zeros((0, 3)), np.float64)
        desc.b_Cf = keep(mesh.b_Cf if self.B else np.zeros((0, 3)), np.float64)
        desc.b_delta_coeffs = keep(mesh.b_delta_coeffs, np.float64)
        pats = (PatchDesc * max(1, len(mesh.patches)))()
        for i, p in enumerate(mesh.patches):
            pats[i].kind = p.kind
            pats[i].is_wall = int(p.is_wall)
            pats[i].p, pats[i].T = p.p, p.T
            for k in range(3):
                pats[i].U[k] = p.U[k]
            pats[i].p0, pats[i].T0 = p.p0, p.T0
            R = p.rotation if p.rotation is not None else (1, 0, 0, 0, 1, 0, 0, 0, 1)
            for k in range(9):
                pats[i].rotation[k] = R[k]
        self._keep.append(pats)
        if mesh.b_partner is not None and np.any(mesh.b_partner >= 0):
            desc.b_partner = keep(mesh.b_partner, np.int32)
            desc.b_weights = keep(mesh.b_weights, np.float64)
            desc.b_nbr_d = keep(mesh.b_nbr_d, np.float64)
            desc.b_nonorth_delta_coeffs = keep(mesh.b_nonorth_delta_coeffs, np.float64)
        desc.patches = pats
        for k in range(3):
            desc.solution_d[k] = mesh.solution_d[k]
        self.cfg = cfg
        h = C.c_void_p()
        st = binding.fn["create"](C.byref(desc), C.byref(cfg), C.byref(h))
        if st != ICS_OK:
            raise IcsError(st, binding.prefix + "create")
        self.h = h

    # ---------------------------------------------------------------- utils
    def _check(self, st: int, where: str, ok=(ICS_OK,)):
        if st not in ok:
            buf = C.create_string_buffer(512)
            if self.h:
                self.b.fn["last_error"](self.h, buf, 512)
            raise IcsError(st, self.b.prefix + where, buf.value.decode(errors="replace"))
        return st

    def close(self):
        if getattr(self, "h", None):
            self.b.fn["destroy"](self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---------------------------------------------------------------- state
    def set_config(self, cfg: Config):
        self.cfg = cfg
        self._check(self.b.fn["set_config"](self.h, C.byref(cfg)), "set_config")

    def set_primitive(self, p, U, T):
        p = np.ascontiguousarray(p, np.float64)
        U = np.ascontiguousarray(U, np.float64).reshape(self.N, 3)
        T = np.ascontiguousarray(T, np.float64)
        self._check(self.b.fn["set_primitive"](self.h, _ptr(p), _ptr(U), _ptr(T)), "set_primitive")

    def set_conservative(self, W, set_old=False):
        W = np.ascontiguousarray(W, np.float64).reshape(self.N, 5)
        self._check(self.b.fn["set_conservative"](self.h, _ptr(W), int(set_old)), "set_conservative")

    def get_state(self):
        W = np.empty((self.N, 5))
        p = np.empty(self.N)
        U = np.empty((self.N, 3))
        T = np.empty(self.N)
        self._check(self.b.fn["get_state"](self.h, _ptr(W), _ptr(p), _ptr(U), _ptr(T)), "get_state")
        return {"W": W, "p": p, "U": U, "T": T}

    def get_conservative(self, out: np.ndarray) -> np.ndarray:
        """Copy the conservative state into ``out`` ([N, 5] float64, C-contiguous, e.g. pinned)."""
        if out.shape != (self.N, 5) or out.dtype != np.float64 or not out.flags.c_contiguous:
            raise ValueError("out must be a C-contiguous float64 [N, 5] array")
        self._check(self.b.fn["get_state"](self.h, _ptr(out), None, None, None), "get_state")
        return out

    def get_boundary_state(self):
        p = np.empty(self.B)
        U = np.empty((self.B, 3))
        T = np.empty(self.B)
        phi = np.empty(self.B)
        self._check(self.b.fn["get_boundary_state"](self.h, _ptr(p), _ptr(U), _ptr(T), _ptr(phi)),
                    "get_boundary_state")
        return {"p": p, "U": U, "T": T, "phi": phi}

    def set_boundary_state(self, p, U, T, phi):
        arrs = [np.ascontiguousarray(a, np.float64) if a is not None else None for a in (p, U, T, phi)]
        self._check(self.b.fn["set_boundary_state"](self.h, *[_ptr(a) for a in arrs]), "set_boundary_state")

    def set_pseudo_co(self, co):
        co = np.ascontiguousarray(np.broadcast_to(co, (self.N,)), np.float64)
        self._check(self.b.fn["set_pseudo_co"](self.h, _ptr(co)), "set_pseudo_co")

    def get_pseudo_co(self):
        co = np.empty(self.N)
        r = np.empty(self.N)
        self._check(self.b.fn["get_pseudo_co"](self.h, _ptr(co), _ptr(r)), "get_pseudo_co")
        return co, r

    # ------------------------------------------------------------- hot path
    def calc_flux(self):
        n = self.F + self.B
        phi = np.empty(n)
        phiU = np.empty((n, 3))
        phiE = np.empty(n)
        self._check(self.b.fn["calc_flux"](self.h, _ptr(phi), _ptr(phiU), _ptr(phiE)), "calc_flux")
        return phi, phiU, phiE

    def residual(self):
        s = np.empty((self.N, 5))
        self._check(self.b.fn["residual"](self.h, _ptr(s)), "residual")
        return s

    def assemble_jacobian(self):
        self._check(self.b.fn["assemble_jacobian"](self.h), "assemble_jacobian")

    def get_jacobian(self):
        d = np.empty((self.N, 5, 5))
        lo = np.empty((self.F, 5, 5))
        up = np.empty((self.F, 5, 5))
        self._check(self.b.fn["get_jacobian"](self.h, _ptr(d), _ptr(lo), _ptr(up)), "get_jacobian")
        return d, lo, up

    def matrix_mul(self, x):
        x = np.ascontiguousarray(x, np.float64).reshape(self.N, 5)
        y = np.empty((self.N, 5))
        self._check(self.b.fn["matrix_mul"](self.h, _ptr(x), _ptr(y)), "matrix_mul")
        return y

    def precondition(self, r):
        r = np.array(r, dtype=np.float64, copy=True).reshape(self.N, 5)
        self._check(self.b.fn["precondition"](self.h, _ptr(r)), "precondition")
        return r

    def solve_increment(self, allow=(ICS_OK,)):
        perf = SolverPerf()
        dW = np.empty((self.N, 5))
        st = self._check(self.b.fn["solve_increment"](self.h, C.byref(perf), _ptr(dW)), "solve_increment", allow)
        return perf, dW, st

    def update_fields(self):
        s = IterStats()
        self._check(self.b.fn["update_fields"](self.h, C.byref(s)), "update_fields")
        return s

    def pseudo_iteration(self):
        s = IterStats()
        self._check(self.b.fn["pseudo_iteration"](self.h, C.byref(s)), "pseudo_iteration")
        return s

    def begin_time_step(self):
        self._check(self.b.fn["begin_time_step"](self.h), "begin_time_step")

    def set_cases(self, case_start):
        """Declare the handle's mesh a stack of independent cases: case k owns
        cells case_start[k] .. case_start[k+1]-1 (see cases.stack_cases)."""
        cs = np.ascontiguousarray(case_start, np.int32)
        self._check(self.b.fn["set_cases"](self.h, len(cs) - 1, _ptr(cs)), "set_cases")
        self.n_cases = len(cs) - 1

    def case_stats(self):
        """Per stacked case: rho L2 residual of the last residual, GMRES
        restart cycles of the last solve, and whether the case is frozen."""
        n = self.n_cases
        l2 = np.zeros(n)
        cyc = np.zeros(n, np.int32)
        fr = np.zeros(n, np.int32)
        self._check(self.b.fn["case_stats"](self.h, _ptr(l2), _ptr(cyc), _ptr(fr)), "case_stats")
        return {"rho_l2": l2, "gmres_cycles": cyc, "frozen": fr.astype(bool)}

    def set_hb(self, n_instances: int, D):
        D = np.ascontiguousarray(D, np.float64).reshape(n_instances, n_instances)
        self._check(self.b.fn["set_hb"](self.h, int(n_instances), _ptr(D)), "set_hb")

    def set_hb_zone(self, zone=None, cyl_coords=False, axis=(0.0, 0.0, 1.0), origin=(0.0, 0.0, 0.0)):
        """HB zone (per-instance cell flags or None for every cell) and cylCoords."""
        z = None if zone is None else np.ascontiguousarray(zone, np.int32)
        a = np.ascontiguousarray(axis, np.float64)
        o = np.ascontiguousarray(origin, np.float64)
        if z is not None:
            self._keep.append(z)
        self._check(self.b.fn["set_hb_zone"](self.h, _ptr(z), int(bool(cyl_coords)), _ptr(a), _ptr(o)),
                    "set_hb_zone")

    def set_phase_lag(self, setup=None):
        """Phase-lag cyclic patches of an HB handle: ``hb.phase_lag_setup``'s
        (mode, P), or None to switch phase lag off."""
        if setup is None:
            self._check(self.b.fn["set_phase_lag"](self.h, None, None), "set_phase_lag")
            return
        mode, P = setup
        mode = np.ascontiguousarray(mode, np.int32)
        P = np.ascontiguousarray(P, np.float64)
        self._keep_plag = (mode, P)
        self._check(self.b.fn["set_phase_lag"](self.h, _ptr(mode), _ptr(P)), "set_phase_lag")

    def set_mrf(self, fields=None, mode: int = 0):
        """Moving reference frames from ``mrf.frame_fields`` (None: off).

        ``fields`` = (omega [N,3], face_velocity [F+B], boundary_U [B,3],
        included [B]); mode 0 = dbnsFoam, 1 = the HB solver's re-assignment
        after every update.
        """
        if fields is None:
            self._check(self.b.fn["set_mrf"](self.h, None, None, None, None, 0), "set_mrf")
            return
        om, fv, bu, inc = fields
        om = np.ascontiguousarray(om, np.float64).reshape(self.N, 3)
        fv = np.ascontiguousarray(fv, np.float64).reshape(-1)
        bu = np.ascontiguousarray(bu, np.float64).reshape(-1, 3)
        inc = np.ascontiguousarray(inc, np.int32).reshape(-1)
        self._keep_mrf = (om, fv, bu, inc)
        self._check(self.b.fn["set_mrf"](self.h, _ptr(om), _ptr(fv), _ptr(bu), _ptr(inc), int(mode)), "set_mrf")

    def pseudo_loop(self) -> bool:
        more = C.c_int32()
        self._check(self.b.fn["pseudo_loop"](self.h, C.byref(more)), "pseudo_loop")
        return bool(more.value)

    # ---------------------------------------------------------- measurement
    def profile(self, enable: bool):
        self._check(self.b.fn["profile"](self.h, int(enable)), "profile")

    def profile_read(self):
        out = {}
        for k, name in enumerate(KERNEL_CLASSES):
            ms = C.c_double()
            n = C.c_int64()
            self._check(self.b.fn["profile_read"](self.h, k, C.byref(ms), C.byref(n)), "profile_read")
            out[name] = (float(ms.value), int(n.value))
        return out

    def launch_count(self) -> int:
        n = C.c_int64()
        self._check(self.b.fn["launch_count"](self.h, C.byref(n)), "launch_count")
        return int(n.value)

    def autotune(self) -> dict:
        """Time the launch choices on this state and keep the fastest (see ics_autotune)."""
        t = Tuning()
        self._check(self.b.fn["autotune"](self.h, C.byref(t)), "autotune")
        return t.as_dict()

    def set_tuning(self, face_block=128, grad_block=128, mgs_blocks=608, fused_operator=1, reverse_rows=1):
        """Apply launch choices (ics_set_tuning), e.g. a saved autotune() result."""
        t = Tuning(face_block=face_block, grad_block=grad_block, mgs_blocks=mgs_blocks,
                   fused_operator=fused_operator, from_cache=0, reverse_rows=reverse_rows)
        self._check(self.b.fn["set_tuning"](self.h, C.byref(t)), "set_tuning")

    def measure_fp64_rate(self) -> float:
        """Measured FP64 FMA rate of the handle's GPU in GFLOP/s."""
        v = C.c_double()
        self._check(self.b.fn["measure_fp64_rate"](self.h, C.byref(v)), "measure_fp64_rate")
        return v.value

    def timer_start(self):
        self._check(self.b.fn["timer_start"](self.h), "timer_start")

    def timer_stop(self) -> float:
        ms = C.c_double()
        self._check(self.b.fn["timer_stop"](self.h, C.byref(ms)), "timer_stop")
        return float(ms.value)

    def test_sweep_timeout(self, skip_row: int, spin_limit: int) -> int:
        """Status of the bounded-wait probe (ICS_ERR_TIMEOUT expected when rows depend on skip_row)."""
        return int(self.b.fn["test_sweep_timeout"](self.h, int(skip_row), int(spin_limit)))

    # ------------------------------------------------- checkpoint / resume
    def save_checkpoint(self) -> bytes:
        n = C.c_int64()
        self._check(self.b.fn["checkpoint_size"](self.h, C.byref(n)), "checkpoint_size")
        buf = C.create_string_buffer(n.value)
        self._check(self.b.fn["save_checkpoint"](self.h, buf, n.value), "save_checkpoint")
        return buf.raw

    def load_checkpoint(self, data: bytes):
        buf = C.create_string_buffer(data, len(data))
        self._check(self.b.fn["load_checkpoint"](self.h, buf, len(data)), "load_checkpoint")

    # ------------------------------------------------------ passive scalar
    def scalar_enable(self, s, patch_fixed=None, patch_value=None, D=0.0, recon=0):
        s = np.ascontiguousarray(np.broadcast_to(s, (self.N,)), np.float64)
        P = len(self.mesh.patches)
        pf = np.ascontiguousarray(np.zeros(P) if patch_fixed is None else patch_fixed, np.int32)
        pv = np.ascontiguousarray(np.zeros(P) if patch_value is None else patch_value, np.float64)
        self._check(self.b.fn["scalar_enable"](self.h, _ptr(s), _ptr(pf), _ptr(pv), float(D), int(recon)),
                    "scalar_enable")

    def scalar_transport(self, n_iterations=1):
        perf = SolverPerf()
        self._check(self.b.fn["scalar_transport"](self.h, int(n_iterations), C.byref(perf)), "scalar_transport")
        return perf

    def get_scalar(self):
        s = np.empty(self.N)
        rs = np.empty(self.N)
        self._check(self.b.fn["get_scalar"](self.h, _ptr(s), _ptr(rs)), "get_scalar")
        return s, rs

    # ------------------------------------------------------ differentiation
    def jvp(self, v: np.ndarray) -> np.ndarray:
        """d(R V)/dW v at the current state (boundary values fixed)."""
        v = np.ascontiguousarray(v, np.float64).reshape(self.N, 5)
        out = np.empty((self.N, 5))
        self._check(self.b.fn["jvp"](self.h, _ptr(v), _ptr(out), 0), "jvp")
        return out

    def vjp(self, u: np.ndarray) -> np.ndarray:
        """(d(R V)/dW)^T u with the exact Jacobian."""
        u = np.ascontiguousarray(u, np.float64).reshape(self.N, 5)
        out = np.empty((self.N, 5))
        self._check(self.b.fn["vjp"](self.h, _ptr(u), _ptr(out), 0), "vjp")
        return out

    def jvp_device(self, v_dev: int, out_dev: int):
        self._check(self.b.fn["jvp"](self.h, v_dev, out_dev, 1), "jvp")

    def vjp_recompute(self, u: np.ndarray) -> np.ndarray:
        """(d(R V)/dW)^T u by reverse mode (no stored Jacobian)."""
        u = np.ascontiguousarray(u, np.float64).reshape(self.N, 5)
        out = np.empty((self.N, 5))
        self._check(self.b.fn["vjp_recompute"](self.h, _ptr(u), _ptr(out), 0), "vjp_recompute")
        return out

    def _krylov(self, fn, rhs, n_directions=30, max_cycles=20, rel_tol=1e-8, precision=0, preconditioner=1,
                pseudo_time=0):
        rhs = np.ascontiguousarray(rhs, np.float64).reshape(self.N, 5)
        sol = np.empty((self.N, 5))
        o = KrylovOpts(n_directions, max_cycles, rel_tol, precision, preconditioner, pseudo_time)
        r = KrylovResult()
        self._check(self.b.fn[fn](self.h, _ptr(rhs), _ptr(sol), C.byref(o), C.byref(r)), fn)
        return sol, r

    def adjoint_solve(self, g, **opts):
        """Solve A^T psi = g, A = pseudo_time V/dtau - d(R V)/dW; returns (psi, KrylovResult)."""
        return self._krylov("adjoint_solve", g, **opts)

    def tangent_solve(self, b, **opts):
        """Solve A x = b, A = pseudo_time V/dtau - d(R V)/dW (matrix-free Newton-Krylov);
        returns (x, KrylovResult)."""
        return self._krylov("tangent_solve", b, **opts)

    def pressure_force(self, patch: int, direction=(1.0, 0.0, 0.0), gradient=True):
        """(J, dJ/dW or None): the patch's integrated pressure force along direction."""
        d = np.ascontiguousarray(direction, np.float64)
        J = C.c_double()
        g = np.empty((self.N, 5)) if gradient else None
        self._check(self.b.fn["pressure_force"](self.h, int(patch), _ptr(d), C.byref(J), _ptr(g)),
                    "pressure_force")
        return J.value, g

    def vjp_device(self, u_dev: int, out_dev: int):
        self._check(self.b.fn["vjp"](self.h, u_dev, out_dev, 1), "vjp")

    def assemble_exact_jacobian(self):
        nnz = C.c_int64()
        ncol = C.c_int32()
        self._check(self.b.fn["assemble_exact_jacobian"](self.h, C.byref(nnz), C.byref(ncol)),
                    "assemble_exact_jacobian")
        return int(nnz.value), int(ncol.value)

    def get_exact_jacobian(self):
        """(row_ptr, cols, blocks[nnz, 5, 5]) of the assembled exact Jacobian."""
        nnz, _ = self._exact_size()
        ptr = np.empty(self.N + 1, np.int32)
        cols = np.empty(nnz, np.int32)
        blocks = np.empty((nnz, 5, 5))
        self._check(self.b.fn["get_exact_jacobian"](self.h, _ptr(ptr), _ptr(cols), _ptr(blocks)),
                    "get_exact_jacobian")
        return ptr, cols, blocks

    def _exact_size(self):
        ptr = np.empty(self.N + 1, np.int32)
        self._check(self.b.fn["get_exact_jacobian"](self.h, _ptr(ptr), None, None), "get_exact_jacobian")
        return int(ptr[-1]), ptr

    def linear_residual_noalloc(self, x_dev: int, r_dev: int, l1_dev: int) -> int:
        """Device-pointer call of ics_linear_residual_noalloc; returns the status."""
        return int(self.b.fn["linear_residual_noalloc"](self.h, x_dev, r_dev, l1_dev))
