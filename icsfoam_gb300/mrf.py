"""Moving reference frames (MRF zones) for the coupled pseudo-time solver.

Host-side set-up of the per-face and per-cell frame quantities the hot path
reads, restated from the reference's zone classes:

* ``MRFCoupledZone`` (``src/cfdTools/MRFCoupled/MRFCoupledZone.C``): a
  rotating cell zone with ``origin``, ``axis``, ``omega`` and optional
  ``nonRotatingPatches``.  ``setMRFFaces`` (:44-229) classifies faces:
  internal faces with either cell in the zone and boundary faces of
  ordinary (non-coupled, non-excluded) patches whose owner is in the zone
  are "included"; faces of coupled or excluded patches whose owner is in the
  zone are "excluded".  ``faceU`` (:544-585) gives Omega x (Cf - origin) on
  the internal, included and excluded faces; ``addOmega`` (:307-318) sets
  Omega on the zone's cells; ``correctBoundaryVelocity`` (:588-613) assigns
  Omega x (Cf - origin) on the included boundary faces.
* ``MRFTranslatingZone`` (``src/cfdTools/MRFTranslating/MRFTranslatingZone.C``):
  a translating cell zone with ``frameVelocity`` and ``nonMovingPatches``;
  the same face classification, a uniform face velocity (:447-482) and the
  same boundary assignment (:485-510).  It has no rotation vector.

dbnsFoam combines them as ``MRFFaceVelocity = MRF.faceU() & Sf/|Sf| +
MRFTrans.faceU() & Sf/|Sf|`` and ``MRFOmega = MRF.omega()``
(``dbnsFoam/outerLoop.H:18-21``), assigning the boundary velocity of the
rotating zones, then of the translating ones (``outerLoop.H:6-7``).
The Harmonic Balance solver sets only ``MRFOmega`` (its face velocity stays
zero, ``dbnsFullyImplicitHBFoam/outerLoop.H:102-105``) and re-assigns the
boundary velocity after every update (``updateFields.H:88``):
``frame_fields(..., harmonic_balance=True)`` returns that combination, for
``CaseHandle.set_mrf(fields, mode=1)``.

Everything here is numpy over the handle's mesh and runs once per case.
"""

from __future__ import annotations

import dataclasses
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

from . import mesh as M

MODE_OUTER_LOOP = 0    # ICS_MRF_OUTER_LOOP
MODE_EVERY_UPDATE = 1  # ICS_MRF_EVERY_UPDATE


def _mask(cells, n: int) -> np.ndarray:
    c = np.asarray(cells)
    if c.dtype == bool:
        if c.shape != (n,):
            raise ValueError("a cell mask must have one entry per cell")
        return c.copy()
    m = np.zeros(n, bool)
    m[c.astype(np.int64)] = True
    return m


@dataclasses.dataclass
class RotatingZone:
    """MRFCoupledZone: ``cells`` (mask or labels), rotation ``omega`` [rad/s]
    about ``axis`` (normalised here, as the reference does) through ``origin``."""

    cells: np.ndarray
    origin: Tuple[float, float, float]
    axis: Tuple[float, float, float]
    omega: float
    non_rotating_patches: Sequence[str] = ()
    active: bool = True
    coupled_patches: Sequence[str] = ()

    def Omega(self) -> np.ndarray:
        a = np.asarray(self.axis, np.float64)
        return self.omega * (a / np.linalg.norm(a))


@dataclasses.dataclass
class TranslatingZone:
    """MRFTranslatingZone: ``cells`` moving with ``frame_velocity`` [m/s]."""

    cells: np.ndarray
    frame_velocity: Tuple[float, float, float]
    non_moving_patches: Sequence[str] = ()
    active: bool = True
    coupled_patches: Sequence[str] = ()


def zone_faces(mesh: M.Mesh, cells, excluded_patches: Sequence[str] = (),
               coupled_patches: Sequence[str] = ()) -> Tuple[np.ndarray, np.ndarray, np.ndarray]:
    """Face classification of setMRFFaces (MRFCoupledZone.C:44-229).

    Returns (internal [F] bool, included [B] bool, excluded [B] bool): internal
    faces with either cell in the zone; boundary faces whose owner is in the
    zone, split by whether their patch is coupled / excluded.  Empty patches
    carry no finite-volume faces here, as they carry none in the reference's
    fvPatch lists.
    """
    zc = _mask(cells, mesh.n_cells)
    internal = zc[mesh.owner] | zc[mesh.neighbour]
    names = [p.name for p in mesh.patches]
    for nm in list(excluded_patches) + list(coupled_patches):
        if nm not in names:
            raise KeyError("unknown patch %r" % nm)
    special = np.array([p.name in excluded_patches or p.name in coupled_patches for p in mesh.patches], bool)
    owner_in = zc[mesh.b_cell] if mesh.n_bfaces else np.zeros(0, bool)
    sp = special[mesh.b_patch] if mesh.n_bfaces else np.zeros(0, bool)
    return internal, owner_in & ~sp, owner_in & sp


def _cross(a, b):
    return np.cross(np.broadcast_to(a, np.shape(b)), b)


def frame_fields(mesh: M.Mesh, rotating: Sequence[RotatingZone] = (), translating: Sequence[TranslatingZone] = (),
                 harmonic_balance: bool = False):
    """(omega [N,3], face_velocity [F+B], boundary_U [B,3], included [B] int32)."""
    N, F, B = mesh.n_cells, mesh.n_faces, mesh.n_bfaces
    n_int = mesh.Sf / np.linalg.norm(mesh.Sf, axis=1)[:, None] if F else np.zeros((0, 3))
    n_b = mesh.b_Sf / np.linalg.norm(mesh.b_Sf, axis=1)[:, None] if B else np.zeros((0, 3))
    omega = np.zeros((N, 3))
    rU_int, rU_b = np.zeros((F, 3)), np.zeros((B, 3))
    tU_int, tU_b = np.zeros((F, 3)), np.zeros((B, 3))
    bU = np.zeros((B, 3))
    inc_all = np.zeros(B, bool)
    for z in rotating:
        if not z.active:
            continue
        Om = z.Omega()
        o = np.asarray(z.origin, np.float64)
        internal, inc, exc = zone_faces(mesh, z.cells, z.non_rotating_patches, z.coupled_patches)
        rU_int[internal] = _cross(Om, mesh.Cf[internal] - o)
        ie = inc | exc
        rU_b[ie] = _cross(Om, mesh.b_Cf[ie] - o)
        omega[_mask(z.cells, N)] = Om
        bU[inc] = _cross(Om, mesh.b_Cf[inc] - o)
        inc_all |= inc
    for z in translating:
        if not z.active:
            continue
        V = np.asarray(z.frame_velocity, np.float64)
        internal, inc, exc = zone_faces(mesh, z.cells, z.non_moving_patches, z.coupled_patches)
        tU_int[internal] = V
        tU_b[inc | exc] = V
        bU[inc] = V
        inc_all |= inc
    fv = np.concatenate([np.einsum("ij,ij->i", rU_int, n_int), np.einsum("ij,ij->i", rU_b, n_b)])
    fv = fv + np.concatenate([np.einsum("ij,ij->i", tU_int, n_int), np.einsum("ij,ij->i", tU_b, n_b)])
    if harmonic_balance:
        fv = np.zeros_like(fv)
    return omega, fv, bU, inc_all.astype(np.int32)


def relative_velocity(mesh: M.Mesh, U: np.ndarray, rotating: Sequence[RotatingZone] = (),
                      translating: Sequence[TranslatingZone] = ()) -> np.ndarray:
    """URel of dbnsFoam (outerLoop.H:9-11): the cell velocity relative to the
    zones' frames (MRFCoupledZone::makeRelative, MRFCoupledZone.C:428-447)."""
    Ur = np.array(U, np.float64, copy=True).reshape(mesh.n_cells, 3)
    for z in rotating:
        if z.active:
            m = _mask(z.cells, mesh.n_cells)
            Ur[m] -= _cross(z.Omega(), mesh.C[m] - np.asarray(z.origin, np.float64))
    for z in translating:
        if z.active:
            m = _mask(z.cells, mesh.n_cells)
            Ur[m] -= np.asarray(z.frame_velocity, np.float64)
    return Ur


def _vec(s: str) -> Tuple[float, float, float]:
    v = [float(x) for x in s.replace("(", " ").replace(")", " ").split()]
    if len(v) != 3:
        raise ValueError("expected a vector, got %r" % s)
    return tuple(v)


def _function1(s: str, n: int):
    """A constant Function1 entry: ``value`` or ``constant value``."""
    t = s.split(None, 1)
    if t and t[0] == "constant":
        s = t[1]
    elif t and not (t[0][0].isdigit() or t[0][0] in "+-.("):
        raise ValueError("only constant Function1 entries are supported, got %r" % s)
    return float(s) if n == 1 else _vec(s)


def _names(s) -> List[str]:
    if not s:
        return []
    return [w.strip('"') for w in str(s).replace("(", " ").replace(")", " ").split()]


def zones_from_dicts(mrf: Optional[Dict], mrf_trans: Optional[Dict], cell_zones: Dict[str, np.ndarray],
                     coupled_patches: Sequence[str] = ()):
    """Zones of constant/MRFProperties and constant/MRFTranslatingProperties
    (one sub-dictionary per zone, MRFCoupledZoneList.C:159-188)."""
    rot, tra = [], []
    for name, d in (mrf or {}).items():
        if not isinstance(d, dict):
            continue
        active = str(d.get("active", "true")).lower() in ("true", "yes", "on", "1")
        cz = d.get("cellZone", name)
        if active and cz not in cell_zones:
            raise KeyError("cannot find MRF cellZone %s" % cz)
        rot.append(RotatingZone(cells=cell_zones.get(cz, np.zeros(0, np.int64)), origin=_vec(d["origin"]),
                                axis=_vec(d["axis"]), omega=_function1(d["omega"], 1),
                                non_rotating_patches=_names(d.get("nonRotatingPatches")), active=active,
                                coupled_patches=tuple(coupled_patches)))
    for name, d in (mrf_trans or {}).items():
        if not isinstance(d, dict):
            continue
        active = str(d.get("active", "true")).lower() in ("true", "yes", "on", "1")
        cz = d.get("cellZone", name)
        if active and cz not in cell_zones:
            raise KeyError("cannot find MRF cellZone %s" % cz)
        tra.append(TranslatingZone(cells=cell_zones.get(cz, np.zeros(0, np.int64)),
                                   frame_velocity=_function1(d["frameVelocity"], 3),
                                   non_moving_patches=_names(d.get("nonMovingPatches")), active=active,
                                   coupled_patches=tuple(coupled_patches)))
    return rot, tra
