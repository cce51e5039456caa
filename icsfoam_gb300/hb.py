"""Harmonic Balance set-up: frequencies, time instants, the spectral operator D
and the stacked multi-instance case.

Restates (host side, tiny dense linear algebra):
* ``omega_list``      HBZone::setOmegaList (HBZone.C:46-92): 0, the positive
  harmonics k*f of every frequency, then the negative ones in reverse order.
* ``find_t0``         HBZoneList::findT0 (HBZoneList.C:32-58): 2 pi / min |omega|.
* ``condition_number`` HBZone::calcConditionN (HBZone.C:195-267): ratio of
  the extreme singular values of E^-1, taken (as the reference does) from
  the eigenvalues of Re(E^-1^H E^-1).
* ``select_instants`` HBZoneList::setInstants (HBZoneList.C:253-346):
  equispaced instants over ``selectedPeriod``, or the period in
  [T0, 5 T0] (steps of 0.001 T0) with the smallest condition number.
* ``hb_operator``     HBZone::updateHBOperators (HBZone.C:270-356):
  E^-1_nk = exp(i omega_k t_n), E = pinv(E^-1), A = diag(omega),
  D = -(Im(E^-1) A Re(E) + Re(E^-1) A Im(E)).
* ``reconstruct``     HBZone::reconstruct (HBZoneTemplates.C:327-405): the
  time history at any t from the instance snapshots (reconstructHBFoam).
* ``phase_lag_operator`` phaseLagCyclicFvPatchField::phaseLaggedField
  (phaseLagCyclicFvPatchFields.C): P = Re(E^-1 M E), M = diag(1, e^{i k
  IBPA} (k = 1..H), e^{-i k IBPA}) -- the instances' values shifted by the
  inter-blade phase angle; ``phase_lag_setup`` lays it out per patch of a
  stacked mesh for ``CaseHandle.set_phase_lag``.

The instances become one stacked mesh (``stack_instances``): instance J owns
cells [J N, (J+1) N) and its own copy of every patch, so time-varying inlet
values differ per instance; the CUDA and oracle libraries couple the same
cell of different instances through D (``ics_set_hb``).
"""

from __future__ import annotations

import copy
from typing import Callable, List, Sequence

import numpy as np

from . import mesh as M


def omega_list(frequencies: Sequence[float], harmonics: Sequence[int]) -> np.ndarray:
    if len(frequencies) != len(harmonics):
        raise ValueError("harmonicsList size must match frequenciesList size")
    pos, neg = [], []
    for f, h in zip(frequencies, harmonics):
        f = abs(f)
        for k in range(1, h + 1):
            pos.append(k * f)
            neg.append(-k * f)
    return np.array([0.0] + pos + neg[::-1])


def find_t0(omegas: np.ndarray) -> float:
    w = np.abs(omegas)
    return 2.0 * np.pi / w[w > 0].min()


def e_inverse(omegas: np.ndarray, instants: np.ndarray) -> np.ndarray:
    return np.exp(1j * np.outer(instants, omegas))


def condition_number(omegas: np.ndarray, instants: np.ndarray) -> float:
    if len(instants) < len(omegas):
        raise ValueError("snapshots size must be equal or greater to omegaList size")
    E1 = e_inverse(omegas, instants)
    G = (E1.conj().T @ E1).real
    ev = np.linalg.eigvals(G).real
    if ev.min() < 1e-15:
        return 1e15
    return float(np.sqrt(ev.max()) / np.sqrt(ev.min()))


def select_instants(omegas: np.ndarray, n_instants: int, selected_period: float = None) -> np.ndarray:
    if selected_period is not None:
        return np.arange(n_instants) * (selected_period / n_instants)
    T0 = find_t0(omegas)
    best, sel = 1e15, None
    Tf = T0
    periods = [T0]
    while Tf <= 5 * T0:
        Tf += 0.001 * T0
        periods.append(Tf)
    for T in periods:
        snaps = (T / n_instants) * np.arange(n_instants)
        c = condition_number(omegas, snaps)
        if c < best:
            best, sel = c, snaps
    return sel


def hb_operator(omegas: np.ndarray, instants: np.ndarray) -> np.ndarray:
    E1 = e_inverse(omegas, instants)
    E = np.linalg.pinv(E1)
    A = np.diag(omegas)
    D = -(E1.imag @ A @ E.real + E1.real @ A @ E.imag)
    return np.ascontiguousarray(D)


def phase_lag_operator(omegas: np.ndarray, instants: np.ndarray, ibpa: float) -> np.ndarray:
    """P[J, K]: the neighbour value of instance J is sum_K P[J, K] f_K."""
    E1 = e_inverse(omegas, instants)
    E = np.linalg.pinv(E1)
    nF = len(omegas)
    nH = (nF - 1) // 2
    Mx = np.zeros((nF, nF), complex)
    Mx[0, 0] = 1.0
    for k in range(1, nH + 1):
        Mx[k, k] = np.exp(1j * k * ibpa)
        Mx[nF - k, nF - k] = np.conj(Mx[k, k])
    return np.ascontiguousarray((E1 @ (Mx @ E)).real)


def phase_lag_setup(mesh: M.Mesh, n: int, omegas: np.ndarray, instants: np.ndarray, ibpa: float,
                    cyl_coords: bool = False, patches: Sequence[str] = None):
    """(mode [n_patches], P [n_patches, n, n]) of a stacked mesh: every cyclic
    patch whose base name is in ``patches`` (all cyclic patches when None)
    becomes phase-lagged; the owner of a pair (the lower patch index, as
    cyclicPolyPatch::owner) takes +IBPA, its neighbour -IBPA."""
    names = [p.name for p in mesh.patches]
    mode = np.zeros(len(names), np.int32)
    P = np.zeros((len(names), n, n))
    for i, p in enumerate(mesh.patches):
        base = p.name.rsplit("_", 1)[0]
        if p.kind != M.PATCH_CYCLIC or (patches is not None and base not in patches):
            continue
        owner = i < names.index(p.partner)
        mode[i] = 2 if cyl_coords else 1
        P[i] = phase_lag_operator(omegas, instants, ibpa if owner else -ibpa)
    return mode, np.ascontiguousarray(P)


def reconstruction_weights(omegas: np.ndarray, instants: np.ndarray, t: float) -> np.ndarray:
    """Weights w_J with f(t) = sum_J w_J f(t_J) for fields band-limited to the
    omega list (HBZone::reconstruct, HBZoneTemplates.C:327-405):
    w = Re(E^-1(t) E) with E^-1(t)_k = exp(i omega_k t) and E = pinv(E^-1)."""
    E = np.linalg.pinv(e_inverse(omegas, instants))
    e1 = np.exp(1j * omegas * t)
    return (e1 @ E).real


def reconstruct(omegas: np.ndarray, instants: np.ndarray, fields: np.ndarray, t: float) -> np.ndarray:
    """A field at time t from its n instance snapshots ``fields`` [n, ...]
    (the reconstructHBFoam post-processing step, one time value)."""
    w = reconstruction_weights(omegas, instants, t)
    return np.tensordot(w, np.asarray(fields), axes=(0, 0))


def stack_instances(mesh: M.Mesh, n: int, patch_for: Callable[[M.Patch, int], M.Patch] = None) -> M.Mesh:
    """n copies of ``mesh`` as one mesh (instance-major cell numbering).

    ``patch_for(patch, J)`` may return a modified copy of a patch for
    instance J (e.g. a time-shifted inlet total pressure).
    """
    N, F, B = mesh.n_cells, mesh.n_faces, mesh.n_bfaces
    P = len(mesh.patches)
    st = copy.copy(mesh)
    st.n_cells = N * n
    off = lambda a, step: np.concatenate([a + J * step for J in range(n)]).astype(a.dtype)
    rep = lambda a: np.concatenate([a] * n)
    st.owner = off(mesh.owner, N)
    st.neighbour = off(mesh.neighbour, N)
    st.Sf, st.Cf, st.weights = rep(mesh.Sf), rep(mesh.Cf), rep(mesh.weights)
    st.delta_coeffs, st.nonorth_delta_coeffs = rep(mesh.delta_coeffs), rep(mesh.nonorth_delta_coeffs)
    st.C, st.V = rep(mesh.C), rep(mesh.V)
    st.b_cell = off(mesh.b_cell, N)
    st.b_Sf, st.b_Cf, st.b_delta_coeffs = rep(mesh.b_Sf), rep(mesh.b_Cf), rep(mesh.b_delta_coeffs)
    st.b_patch = off(mesh.b_patch, P)
    if mesh.b_partner is not None:
        st.b_partner = np.concatenate([np.where(mesh.b_partner >= 0, mesh.b_partner + J * N, -1)
                                       for J in range(n)]).astype(np.int32)
        st.b_weights, st.b_nbr_d = rep(mesh.b_weights), rep(mesh.b_nbr_d)
        st.b_nonorth_delta_coeffs = rep(mesh.b_nonorth_delta_coeffs)
    pats: List[M.Patch] = []
    for J in range(n):
        for p in mesh.patches:
            q = copy.copy(p)
            q.name = "%s_%d" % (p.name, J)
            if q.partner is not None:
                q.partner = "%s_%d" % (p.partner, J)
            pats.append(patch_for(q, J) if patch_for else q)
    st.patches = pats
    st.cell_ijk = rep(mesh.cell_ijk) if mesh.cell_ijk is not None else None
    st.points = st.face_points = st.b_face_points = None
    return st
