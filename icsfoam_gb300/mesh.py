"""Host-side mesh construction for the coupled pseudo-time solver.

Builds OpenFOAM-convention finite-volume meshes (owner < neighbour, internal
faces in upper-triangular order, boundary faces grouped by patch, empty
patches dropped from the finite-volume addressing) and the geometric
quantities the reference path reads from ``fvMesh``:

* face area vectors ``Sf`` and centres ``Cf`` (triangle decomposition about
  the face's average point),
* cell centres ``C`` and volumes ``V`` (pyramid decomposition about the
  average of the face centres),
* interpolation ``weights``, ``deltaCoeffs`` and ``nonOrthDeltaCoeffs``.

The reference reads all of these from OpenFOAM v2112 (for example
``convectiveFluxScheme.C:65,376,411``, ``setCoAndDeltaT.H:61,93`` and
``blockFvOperatorsTemplates.C:408-409``); OpenFOAM is a third-party
dependency absent here, so the formulas below restate its documented
geometry (primitiveMesh face/cell centre algorithms, surfaceInterpolation
weights and delta coefficients).

Everything here is plain numpy and runs once per mesh, outside the timed
path.  Cell renumbering (RCM, colour blocking) lives in ``ordering.py``.
"""

from __future__ import annotations

import dataclasses
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

# Patch kinds understood by the C-ABI (must match include/icsfoam_gb300.h).
PATCH_ZERO_GRADIENT = 1    # U, p, T zeroGradient
PATCH_SLIP = 2             # U slip, p/T zeroGradient
PATCH_FIXED = 3            # U, p, T fixedValue
PATCH_PRESSURE_OUTLET = 4  # p fixedValue, U/T zeroGradient
PATCH_TOTAL_INLET = 5      # totalPressure / totalTemperature / pressureInletOutletVelocity
PATCH_ISOTHERMAL_WALL = 6  # U fixed 0, T fixed, p zeroGradient
PATCH_CYCLIC = 7           # coupled to a partner patch, face i <-> face i (rotational or parallel)
PATCH_EMPTY = 0            # no finite-volume faces

PATCH_NAMES = {
    "zeroGradient": PATCH_ZERO_GRADIENT,
    "slip": PATCH_SLIP,
    "fixedValue": PATCH_FIXED,
    "pressureOutlet": PATCH_PRESSURE_OUTLET,
    "totalInlet": PATCH_TOTAL_INLET,
    "isothermalWall": PATCH_ISOTHERMAL_WALL,
    "cyclic": PATCH_CYCLIC,
    "empty": PATCH_EMPTY,
}

ROOTVSMALL = 1.0e-150
VSMALL = 1.0e-300


@dataclasses.dataclass
class Patch:
    """One boundary patch: a BC kind plus its fixed values.

    ``is_wall`` marks OpenFOAM ``wall``-type patches, which the local pseudo
    time step treats specially (``setCoAndDeltaT.H:88-136``).

    A cyclic patch (``kind == PATCH_CYCLIC``) names its ``partner`` patch;
    face i of the two is one coupled face.  ``rotation`` (row-major 3x3)
    maps vectors of the partner's side into this patch's frame (OpenFOAM
    cyclic forwardT; the identity for a parallel cyclic), ``centre`` is the
    point it rotates about (used to check the face pairing).
    """

    name: str
    kind: int
    is_wall: bool = False
    p: float = 0.0
    T: float = 0.0
    U: Tuple[float, float, float] = (0.0, 0.0, 0.0)
    p0: float = 0.0
    T0: float = 0.0
    partner: Optional[str] = None
    rotation: Optional[Tuple[float, ...]] = None
    centre: Tuple[float, float, float] = (0.0, 0.0, 0.0)
    separation: Tuple[float, float, float] = (0.0, 0.0, 0.0)


def rotation_matrix(axis, angle_deg: float) -> np.ndarray:
    """Right-handed rotation by ``angle_deg`` about ``axis`` (Rodrigues)."""
    a = np.asarray(axis, np.float64)
    a = a / np.linalg.norm(a)
    t = np.radians(angle_deg)
    K = np.array([[0, -a[2], a[1]], [a[2], 0, -a[0]], [-a[1], a[0], 0]])
    return np.eye(3) + np.sin(t) * K + (1.0 - np.cos(t)) * (K @ K)


def cyclic_pair(name_a: str, name_b: str, axis=(0.0, 0.0, 1.0), angle_deg: float = 0.0,
                centre=(0.0, 0.0, 0.0), separation=(0.0, 0.0, 0.0)) -> Tuple[Patch, Patch]:
    """Two coupled patches: rotating patch b's geometry by ``angle_deg`` about
    ``axis`` through ``centre`` and shifting it by ``separation`` lands it on
    patch a (a rotational cyclic, or a translational one at 0 degrees)."""
    R = rotation_matrix(axis, angle_deg)
    sep = np.asarray(separation, np.float64)
    a = Patch(name_a, PATCH_CYCLIC, partner=name_b, rotation=tuple(R.ravel()), centre=tuple(centre),
              separation=tuple(sep))
    b = Patch(name_b, PATCH_CYCLIC, partner=name_a, rotation=tuple(R.T.ravel()), centre=tuple(centre),
              separation=tuple(-(R.T @ sep)))
    return a, b


@dataclasses.dataclass
class Mesh:
    """Finite-volume mesh in OpenFOAM LDU convention.

    Arrays are float64 / int32, C-contiguous, vectors stored as (n, 3).
    """

    n_cells: int
    owner: np.ndarray          # (F,) int32, internal faces
    neighbour: np.ndarray      # (F,) int32
    Sf: np.ndarray             # (F, 3)
    Cf: np.ndarray             # (F, 3)
    weights: np.ndarray        # (F,)
    delta_coeffs: np.ndarray   # (F,)
    nonorth_delta_coeffs: np.ndarray  # (F,)
    C: np.ndarray              # (N, 3)
    V: np.ndarray              # (N,)
    b_cell: np.ndarray         # (B,) int32
    b_Sf: np.ndarray           # (B, 3)
    b_Cf: np.ndarray           # (B, 3)
    b_delta_coeffs: np.ndarray  # (B,)
    b_patch: np.ndarray        # (B,) int32
    patches: List[Patch]
    solution_d: Tuple[int, int, int]
    # Topology kept for renumbering (internal + non-empty boundary faces).
    points: Optional[np.ndarray] = None
    face_points: Optional[np.ndarray] = None     # (F, 4) internal faces
    b_face_points: Optional[np.ndarray] = None   # (B, 4)
    cell_ijk: Optional[np.ndarray] = None        # (N, 3) generator index
    # coupled (cyclic) boundary faces: the partner patch's cell of the paired
    # face (-1 elsewhere), linear weight, the vector from the partner cell's
    # centre (in this side's frame) to the face centre, nonOrthDeltaCoeffs
    b_partner: Optional[np.ndarray] = None       # (B,) int32
    b_weights: Optional[np.ndarray] = None       # (B,)
    b_nbr_d: Optional[np.ndarray] = None         # (B, 3)
    b_nonorth_delta_coeffs: Optional[np.ndarray] = None  # (B,)

    @property
    def n_faces(self) -> int:
        return int(self.owner.shape[0])

    @property
    def n_bfaces(self) -> int:
        return int(self.b_cell.shape[0])

    def patch_range(self, name: str) -> np.ndarray:
        idx = [i for i, p in enumerate(self.patches) if p.name == name]
        if not idx:
            raise KeyError(name)
        return np.nonzero(self.b_patch == idx[0])[0]


# --------------------------------------------------------------------------
# Geometry (restated from OpenFOAM primitiveMesh / surfaceInterpolation)
# --------------------------------------------------------------------------

def face_centres_and_areas(points: np.ndarray, fp) -> Tuple[np.ndarray, np.ndarray]:
    """Face centres and area vectors by triangle decomposition.

    Each polygon is split into triangles about its average point; the area
    vector is half the sum of the triangle normals and the centre is the
    area-weighted mean of the triangle centroids.  ``fp`` is an (n, k) array
    of point labels, or an object array of label arrays of mixed sizes.
    """
    if fp.dtype == object:
        Cf = np.zeros((len(fp), 3))
        Sf = np.zeros((len(fp), 3))
        sizes = np.array([len(f) for f in fp])
        for k in np.unique(sizes):
            idx = np.nonzero(sizes == k)[0]
            c, s = face_centres_and_areas(points, np.stack([fp[i] for i in idx]).astype(np.int64))
            Cf[idx] = c
            Sf[idx] = s
        return Cf, Sf
    P = points[fp]                       # (nF, k, 3)
    fc = P.mean(axis=1)                  # average point
    sumN = np.zeros_like(fc)
    sumA = np.zeros(fc.shape[0])
    sumAc = np.zeros_like(fc)
    nv = fp.shape[1]
    for pi in range(nv):
        a = P[:, pi]
        b = P[:, (pi + 1) % nv]
        c = a + b + fc
        n = np.cross(b - a, fc - a)
        an = np.linalg.norm(n, axis=1)
        sumN += n
        sumA += an
        sumAc += an[:, None] * c
    small = sumA < ROOTVSMALL
    Cf = np.where(small[:, None], fc, (1.0 / 3.0) * sumAc / np.where(small, 1.0, sumA)[:, None])
    Sf = 0.5 * sumN
    return Cf, Sf


def cell_centres_and_volumes(n_cells: int, own: np.ndarray, nei: np.ndarray, Cf: np.ndarray,
                             Sf: np.ndarray, b_cell: np.ndarray, b_Cf: np.ndarray,
                             b_Sf: np.ndarray, extra_cell: np.ndarray = None,
                             extra_Cf: np.ndarray = None, extra_Sf: np.ndarray = None
                             ) -> Tuple[np.ndarray, np.ndarray]:
    """Cell centres and volumes by pyramid decomposition.

    The estimated centre is the average of the cell's face centres; every
    face forms a pyramid with it.  ``extra_*`` are faces that bound cells but
    are not finite-volume faces (empty patches) - they still enclose volume.
    """
    allc = [own, nei, b_cell]
    allCf = [Cf, Cf, b_Cf]
    if extra_cell is not None and len(extra_cell):
        allc.append(extra_cell)
        allCf.append(extra_Cf)
    nf = np.zeros(n_cells)
    cEst = np.zeros((n_cells, 3))
    for c, cf in zip(allc, allCf):
        np.add.at(nf, c, 1.0)
        np.add.at(cEst, c, cf)
    cEst /= nf[:, None]

    vol = np.zeros(n_cells)
    ctr = np.zeros((n_cells, 3))

    def acc(cells, cf, sf, sign):
        pyr3 = np.maximum(sign * np.einsum("ij,ij->i", sf, cf - cEst[cells]), VSMALL)
        pc = 0.75 * cf + 0.25 * cEst[cells]
        np.add.at(ctr, cells, pyr3[:, None] * pc)
        np.add.at(vol, cells, pyr3)

    acc(own, Cf, Sf, 1.0)
    acc(nei, Cf, Sf, -1.0)
    acc(b_cell, b_Cf, b_Sf, 1.0)
    if extra_cell is not None and len(extra_cell):
        acc(extra_cell, extra_Cf, extra_Sf, 1.0)
    good = np.abs(vol) > VSMALL
    C = np.where(good[:, None], ctr / np.where(good, vol, 1.0)[:, None], cEst)
    V = vol * (1.0 / 3.0)
    return C, V


def interpolation_coeffs(own, nei, Sf, Cf, C, b_cell, b_Sf, b_Cf):
    """weights, deltaCoeffs, nonOrthDeltaCoeffs for internal and boundary faces."""
    magSf = np.linalg.norm(Sf, axis=1)
    SfdOwn = np.abs(np.einsum("ij,ij->i", Sf, Cf - C[own]))
    SfdNei = np.abs(np.einsum("ij,ij->i", Sf, C[nei] - Cf))
    w = SfdNei / (SfdOwn + SfdNei)
    delta = C[nei] - C[own]
    dc = 1.0 / np.linalg.norm(delta, axis=1)
    unit = Sf / magSf[:, None]
    nodc = 1.0 / np.maximum(np.einsum("ij,ij->i", unit, delta), 0.05 * np.linalg.norm(delta, axis=1))
    # non-coupled boundary: delta is the normal projection of Cf - C
    bmag = np.linalg.norm(b_Sf, axis=1)
    bn = b_Sf / bmag[:, None]
    bd = np.abs(np.einsum("ij,ij->i", bn, b_Cf - C[b_cell]))
    bdc = 1.0 / bd
    return w, dc, nodc, bdc


# --------------------------------------------------------------------------
# Structured hex generator
# --------------------------------------------------------------------------

SIDES = ("xmin", "xmax", "ymin", "ymax", "zmin", "zmax")


def hex_mesh(points_grid: np.ndarray, side_patches: Dict[str, Patch],
             side_split: Optional[Dict[str, Sequence[Tuple[Patch, np.ndarray]]]] = None) -> Mesh:
    """Build a hex mesh from a (nx+1, ny+1, nz+1, 3) grid of points.

    ``side_patches`` maps each of the six sides to a Patch; patches of kind
    PATCH_EMPTY are dropped from the finite-volume faces (OpenFOAM empty).
    ``side_split`` optionally splits a side into several patches by a mask
    over that side's faces (the mask is indexed like the side's 2D face grid).
    Cell index = i + nx*(j + ny*k).
    """
    nxp, nyp, nzp, _ = points_grid.shape
    nx, ny, nz = nxp - 1, nyp - 1, nzp - 1
    pts = points_grid.transpose(2, 1, 0, 3).reshape(-1, 3).copy()

    def pid(i, j, k):
        return i + nxp * (j + nyp * k)

    def cid(i, j, k):
        return i + nx * (j + ny * k)

    faces = []  # list of (points(4), owner, neighbour or -1, side or None, side-local index)

    # x faces
    I, J, K = np.meshgrid(np.arange(nx + 1), np.arange(ny), np.arange(nz), indexing="ij")
    fx = np.stack([pid(I, J, K), pid(I, J + 1, K), pid(I, J + 1, K + 1), pid(I, J, K + 1)], axis=-1)
    # y faces
    I2, J2, K2 = np.meshgrid(np.arange(nx), np.arange(ny + 1), np.arange(nz), indexing="ij")
    fy = np.stack([pid(I2, J2, K2), pid(I2, J2, K2 + 1), pid(I2 + 1, J2, K2 + 1), pid(I2 + 1, J2, K2)], axis=-1)
    # z faces
    I3, J3, K3 = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz + 1), indexing="ij")
    fz = np.stack([pid(I3, J3, K3), pid(I3 + 1, J3, K3), pid(I3 + 1, J3 + 1, K3), pid(I3, J3 + 1, K3)], axis=-1)

    int_pts, int_own, int_nei = [], [], []
    # internal x faces: owner (i-1), neighbour (i)
    int_pts.append(fx[1:nx].reshape(-1, 4))
    int_own.append(cid(I[1:nx] - 1, J[1:nx], K[1:nx]).ravel())
    int_nei.append(cid(I[1:nx], J[1:nx], K[1:nx]).ravel())
    int_pts.append(fy[:, 1:ny].reshape(-1, 4))
    int_own.append(cid(I2[:, 1:ny], J2[:, 1:ny] - 1, K2[:, 1:ny]).ravel())
    int_nei.append(cid(I2[:, 1:ny], J2[:, 1:ny], K2[:, 1:ny]).ravel())
    int_pts.append(fz[:, :, 1:nz].reshape(-1, 4))
    int_own.append(cid(I3[:, :, 1:nz], J3[:, :, 1:nz], K3[:, :, 1:nz] - 1).ravel())
    int_nei.append(cid(I3[:, :, 1:nz], J3[:, :, 1:nz], K3[:, :, 1:nz]).ravel())
    fp_int = np.concatenate(int_pts)
    own = np.concatenate(int_own).astype(np.int64)
    nei = np.concatenate(int_nei).astype(np.int64)

    # boundary sides: (points with outward normal, owner cell, 2D shape)
    side_faces = {
        "xmin": (fx[0][..., ::-1], cid(np.zeros_like(J[0]), J[0], K[0])),
        "xmax": (fx[nx], cid(np.full_like(J[0], nx - 1), J[0], K[0])),
        "ymin": (fy[:, 0][..., ::-1], cid(I2[:, 0], np.zeros_like(I2[:, 0]), K2[:, 0])),
        "ymax": (fy[:, ny], cid(I2[:, 0], np.full_like(I2[:, 0], ny - 1), K2[:, 0])),
        "zmin": (fz[:, :, 0][..., ::-1], cid(I3[:, :, 0], J3[:, :, 0], np.zeros_like(I3[:, :, 0]))),
        "zmax": (fz[:, :, nz], cid(I3[:, :, 0], J3[:, :, 0], np.full_like(I3[:, :, 0], nz - 1))),
    }
    # order patches: unique Patch objects in first-appearance order over sides
    patch_list: List[Patch] = []
    entries = []  # (patch, fp(n,4), cells(n))
    for side in SIDES:
        fps, cells = side_faces[side]
        fps = fps.reshape(-1, 4)
        cells = cells.ravel()
        if side_split and side in side_split:
            for patch, mask in side_split[side]:
                m = np.asarray(mask).ravel()
                entries.append((patch, fps[m], cells[m]))
        else:
            entries.append((side_patches[side], fps, cells))
    for patch, _, _ in entries:
        if all(patch is not q for q in patch_list):
            patch_list.append(patch)

    return _finish(pts, fp_int, own, nei, entries, patch_list, (nx, ny, nz))


def _finish(pts, fp_int, own, nei, entries, patch_list, dims=None, cell_ijk=None) -> Mesh:
    n_cells = int(max(own.max(initial=-1), nei.max(initial=-1)) + 1)
    for _, _, cells in entries:
        if len(cells):
            n_cells = max(n_cells, int(cells.max()) + 1)
    # upper-triangular order
    order = np.lexsort((nei, own))
    fp_int, own, nei = fp_int[order], own[order], nei[order]

    fv_patches = [p for p in patch_list if p.kind != PATCH_EMPTY]
    b_fp, b_cell, b_patch = [], [], []
    e_fp, e_cell = [], []
    for pi, patch in enumerate(fv_patches):
        for p, fps, cells in entries:
            if p is patch:
                b_fp.append(fps)
                b_cell.append(cells)
                b_patch.append(np.full(len(cells), pi))
    for p, fps, cells in entries:
        if p.kind == PATCH_EMPTY:
            e_fp.append(fps)
            e_cell.append(cells)
    b_fp = np.concatenate(b_fp) if b_fp else np.zeros((0, 4), np.int64)
    b_cell = np.concatenate(b_cell).astype(np.int64) if b_cell else np.zeros(0, np.int64)
    b_patch = np.concatenate(b_patch) if b_patch else np.zeros(0, np.int64)
    e_fp = np.concatenate(e_fp) if e_fp else np.zeros((0, 4), np.int64)
    e_cell = np.concatenate(e_cell).astype(np.int64) if e_cell else np.zeros(0, np.int64)

    Cf, Sf = face_centres_and_areas(pts, fp_int)
    bCf, bSf = face_centres_and_areas(pts, b_fp) if len(b_fp) else (np.zeros((0, 3)), np.zeros((0, 3)))
    eCf, eSf = face_centres_and_areas(pts, e_fp) if len(e_fp) else (np.zeros((0, 3)), np.zeros((0, 3)))
    C, V = cell_centres_and_volumes(n_cells, own, nei, Cf, Sf, b_cell, bCf, bSf, e_cell, eCf, eSf)
    w, dc, nodc, bdc = interpolation_coeffs(own, nei, Sf, Cf, C, b_cell, bSf, bCf)

    # solution directions: a direction is unsolved if empty patches span it
    sol = [1, 1, 1]
    if len(e_fp):
        en = eSf / np.linalg.norm(eSf, axis=1)[:, None]
        emax = np.abs(en).max(axis=0)
        for d in range(3):
            if emax[d] > 0.5:
                sol[d] = -1
    cyc = cyclic_geometry(fv_patches, b_patch, b_cell, bSf, bCf, C)
    m = Mesh(
        n_cells=n_cells,
        owner=own.astype(np.int32), neighbour=nei.astype(np.int32),
        Sf=np.ascontiguousarray(Sf), Cf=np.ascontiguousarray(Cf),
        weights=w, delta_coeffs=dc, nonorth_delta_coeffs=nodc,
        C=np.ascontiguousarray(C), V=V,
        b_cell=b_cell.astype(np.int32), b_Sf=np.ascontiguousarray(bSf), b_Cf=np.ascontiguousarray(bCf),
        b_delta_coeffs=bdc, b_patch=b_patch.astype(np.int32),
        patches=fv_patches, solution_d=tuple(sol),
        points=pts, face_points=fp_int, b_face_points=b_fp,
    )
    m.b_partner, m.b_weights, m.b_nbr_d, cyc_dc, cyc_nodc = cyc
    m.b_nonorth_delta_coeffs = m.b_delta_coeffs.copy()
    sel = m.b_partner >= 0
    m.b_delta_coeffs[sel] = cyc_dc[sel]
    m.b_nonorth_delta_coeffs[sel] = cyc_nodc[sel]
    m._empty = (e_fp, e_cell)  # kept for renumbering
    if cell_ijk is not None:
        m.cell_ijk = cell_ijk
    elif dims is not None:
        nx, ny, nz = dims
        c = np.arange(n_cells)
        m.cell_ijk = np.stack([c % nx, (c // nx) % ny, c // (nx * ny)], axis=1).astype(np.int32)
    return m


def cyclic_geometry(patches: List[Patch], b_patch, b_cell, bSf, bCf, C):
    """Coupled-face data of cyclic patches (OpenFOAM cyclicFvPatch):

    * partner cell: owner of face i of the partner patch;
    * weights w = dn / (d + dn), d = n . (Cf - C_own) on this side and dn the
      same on the partner side (cyclicFvPatch::makeWeights);
    * delta = (Cf - C_own) - R (Cf_nbr - C_nbr) (cyclicFvPatch::delta), so the
      partner centre seen from this side is C_own + delta; deltaCoeffs =
      1/|delta|, nonOrthDeltaCoeffs = 1/max(n . delta, 0.05 |delta|);
    * nbr_d = Cf - (C_own + delta): the partner-side displacement that
      linearUpwind extrapolates along.
    Face pairing is checked: R (Cf_nbr - centre) + centre + separation must
    land on Cf.
    """
    B = len(b_patch)
    partner = np.full(B, -1, np.int32)
    w = np.ones(B)
    nbr_d = np.zeros((B, 3))
    dc = np.zeros(B)
    nodc = np.zeros(B)
    names = [p.name for p in patches]
    for pi, p in enumerate(patches):
        if p.kind != PATCH_CYCLIC:
            continue
        if p.partner not in names:
            raise ValueError("cyclic patch %s: partner %r not found" % (p.name, p.partner))
        qi = names.index(p.partner)
        q = patches[qi]
        if q.kind != PATCH_CYCLIC or q.partner != p.name:
            raise ValueError("cyclic patches %s and %s do not name each other" % (p.name, q.name))
        fa = np.nonzero(b_patch == pi)[0]
        fb = np.nonzero(b_patch == qi)[0]
        if len(fa) != len(fb):
            raise ValueError("cyclic patches %s and %s differ in size" % (p.name, q.name))
        R = np.asarray(p.rotation if p.rotation is not None else np.eye(3).ravel(), np.float64).reshape(3, 3)
        ctr = np.asarray(p.centre, np.float64)
        mapped = (bCf[fb] - ctr) @ R.T + ctr + np.asarray(p.separation, np.float64)
        # OpenFOAM's matchTolerance: a fraction of the face length scale
        tol = getattr(p, "match_tolerance", 1e-4) * np.sqrt(np.linalg.norm(bSf[fa], axis=1))
        if len(fa) and np.any(np.abs(mapped - bCf[fa]).max(axis=1) > tol):
            raise ValueError("cyclic patches %s and %s: faces do not pair under the rotation" % (p.name, q.name))
        na = bSf[fa] / np.linalg.norm(bSf[fa], axis=1)[:, None]
        nb = bSf[fb] / np.linalg.norm(bSf[fb], axis=1)[:, None]
        da = bCf[fa] - C[b_cell[fa]]
        db = bCf[fb] - C[b_cell[fb]]
        di = np.einsum("ij,ij->i", na, da)
        dni = np.einsum("ij,ij->i", nb, db)
        partner[fa] = b_cell[fb]
        w[fa] = dni / (di + dni)
        delta = da - db @ R.T
        nbr_d[fa] = da - delta
        md = np.linalg.norm(delta, axis=1)
        dc[fa] = 1.0 / md
        nodc[fa] = 1.0 / np.maximum(np.einsum("ij,ij->i", na, delta), 0.05 * md)
    return partner, w, nbr_d, dc, nodc


def renumber(mesh: Mesh, new_to_old: np.ndarray) -> Mesh:
    """Renumber cells (``new_to_old[n]`` = old index of new cell n).

    Faces are re-oriented so that owner < neighbour and re-sorted into
    upper-triangular order; geometry is recomputed from the points, exactly
    as OpenFOAM's renumberMesh leaves a valid LDU mesh behind.
    """
    new_to_old = np.asarray(new_to_old, dtype=np.int64)
    old_to_new = np.empty_like(new_to_old)
    old_to_new[new_to_old] = np.arange(len(new_to_old))
    own = old_to_new[mesh.owner.astype(np.int64)]
    nei = old_to_new[mesh.neighbour.astype(np.int64)]
    fp = mesh.face_points.copy()
    flip = own > nei
    if fp.dtype == object:
        for i in np.nonzero(flip)[0]:
            fp[i] = fp[i][::-1]
    else:
        fp[flip] = fp[flip][:, ::-1]
    o2 = np.where(flip, nei, own)
    n2 = np.where(flip, own, nei)
    entries = []
    for pi, patch in enumerate(mesh.patches):
        sel = mesh.b_patch == pi
        entries.append((patch, mesh.b_face_points[sel], old_to_new[mesh.b_cell[sel].astype(np.int64)]))
    e_fp, e_cell = mesh._empty
    empty_patch = Patch("empty", PATCH_EMPTY)
    if len(e_fp):
        entries.append((empty_patch, e_fp, old_to_new[e_cell]))
    plist = list(mesh.patches) + ([empty_patch] if len(e_fp) else [])
    ijk = mesh.cell_ijk[new_to_old] if mesh.cell_ijk is not None else None
    m = _finish(mesh.points, fp, o2, n2, entries, plist, cell_ijk=ijk)
    return m


def cell_faces_csr(mesh: Mesh) -> Tuple[np.ndarray, np.ndarray]:
    """CSR cell -> internal faces (encoded f for owner side, ~f for neighbour side).

    Within a cell the faces are listed in increasing face index, which is the
    order OpenFOAM's ``cells()`` lists them for an upper-triangular mesh
    closely enough for every consumer here (all consumers are order-free
    sums or use the explicit lower/upper split).
    """
    F = mesh.n_faces
    cells = np.concatenate([mesh.owner, mesh.neighbour]).astype(np.int64)
    codes = np.concatenate([np.arange(F), ~np.arange(F)]).astype(np.int64)
    faces = np.concatenate([np.arange(F), np.arange(F)])
    order = np.lexsort((faces, cells))
    ptr = np.zeros(mesh.n_cells + 1, np.int64)
    np.add.at(ptr, cells + 1, 1)
    ptr = np.cumsum(ptr)
    return ptr.astype(np.int32), codes[order].astype(np.int32)


def stack(meshes: Sequence[Mesh]) -> Tuple[Mesh, np.ndarray]:
    """The disjoint union of independent meshes as one mesh (case-major cell
    numbering: mesh k's cells follow those of meshes 0..k-1, each in its own
    order) and the case offsets start[k] (n_cases + 1 entries).  Each mesh's
    patches are kept as patches of their own, named ``<name>_<k>``; internal
    faces keep each mesh's order, so the owner-ordered face list and every
    cell's face order are those of the mesh alone."""
    if not meshes:
        raise ValueError("no meshes to stack")
    sd = meshes[0].solution_d
    if any(m.solution_d != sd for m in meshes):
        raise ValueError("stacked meshes must share their solution directions")
    if any(m.b_partner is not None and np.any(m.b_partner >= 0) for m in meshes):
        raise ValueError("stacked meshes carry no cyclic patches")
    start = np.zeros(len(meshes) + 1, np.int32)
    start[1:] = np.cumsum([m.n_cells for m in meshes])
    poff = np.cumsum([0] + [len(m.patches) for m in meshes])
    cat = lambda f: np.concatenate([f(m) for m in meshes])
    pats: List[Patch] = []
    for k, m in enumerate(meshes):
        for p in m.patches:
            q = dataclasses.replace(p, name="%s_%d" % (p.name, k))
            pats.append(q)
    st = dataclasses.replace(
        meshes[0],
        n_cells=int(start[-1]),
        owner=np.concatenate([m.owner + start[k] for k, m in enumerate(meshes)]).astype(np.int32),
        neighbour=np.concatenate([m.neighbour + start[k] for k, m in enumerate(meshes)]).astype(np.int32),
        Sf=cat(lambda m: m.Sf), Cf=cat(lambda m: m.Cf), weights=cat(lambda m: m.weights),
        delta_coeffs=cat(lambda m: m.delta_coeffs), nonorth_delta_coeffs=cat(lambda m: m.nonorth_delta_coeffs),
        C=cat(lambda m: m.C), V=cat(lambda m: m.V),
        b_cell=np.concatenate([m.b_cell + start[k] for k, m in enumerate(meshes)]).astype(np.int32),
        b_Sf=cat(lambda m: m.b_Sf), b_Cf=cat(lambda m: m.b_Cf), b_delta_coeffs=cat(lambda m: m.b_delta_coeffs),
        b_patch=np.concatenate([m.b_patch + poff[k] for k, m in enumerate(meshes)]).astype(np.int32),
        patches=pats, points=None, face_points=None, b_face_points=None, cell_ijk=None, b_partner=None,
        b_weights=None, b_nbr_d=None, b_nonorth_delta_coeffs=None)
    return st, start
