"""Cell orderings: natural, reverse Cuthill-McKee, colour-blocked.

LU-SGS (lusgs.C:220-385) sweeps cells in their numbering.  The GPU runs it
level by level: a level holds cells whose lower (forward) or upper (reverse)
neighbours all lie in earlier levels.  Under the natural numbering of a
structured nx*ny*nz box that is nx+ny+nz-2 levels; under the colour-blocked
numbering built here (cells sorted by greedy colour, then by old index) it is
one level per colour, typically 2 for hex meshes.  The oracle runs the
reference's sequential sweep on the same numbering, so both variants keep
exact algorithmic parity - renumbering only changes which preconditioner
the reference itself would have applied to the renumbered mesh.
"""

from __future__ import annotations

import ctypes as C

import numpy as np

from . import _build
from . import mesh as M

_HOST = None


def host_lib():
    global _HOST
    if _HOST is None:
        lib = C.CDLL(_build.build_host())
        lib.ics_mesh_greedy_colour.restype = C.c_int32
        lib.ics_mesh_greedy_colour.argtypes = [C.c_int32, C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p]
        lib.ics_mesh_rcm.restype = C.c_int32
        lib.ics_mesh_rcm.argtypes = [C.c_int32, C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p]
        _HOST = lib
    return _HOST


def greedy_colour(mesh: M.Mesh):
    own = np.ascontiguousarray(mesh.owner, np.int32)
    nei = np.ascontiguousarray(mesh.neighbour, np.int32)
    col = np.empty(mesh.n_cells, np.int32)
    n = host_lib().ics_mesh_greedy_colour(mesh.n_cells, own.ctypes.data, nei.ctypes.data, mesh.n_faces,
                                          col.ctypes.data)
    if n < 0:
        raise ValueError("colouring failed")
    return col, int(n)


def rcm(mesh: M.Mesh) -> np.ndarray:
    own = np.ascontiguousarray(mesh.owner, np.int32)
    nei = np.ascontiguousarray(mesh.neighbour, np.int32)
    out = np.empty(mesh.n_cells, np.int32)
    if host_lib().ics_mesh_rcm(mesh.n_cells, own.ctypes.data, nei.ctypes.data, mesh.n_faces, out.ctypes.data):
        raise ValueError("rcm failed")
    return out


def colour_blocked(mesh: M.Mesh) -> np.ndarray:
    col, _ = greedy_colour(mesh)
    return np.lexsort((np.arange(mesh.n_cells), col)).astype(np.int64)


def permutation(mesh: M.Mesh, mode: str) -> np.ndarray:
    """new_to_old cell permutation of an ordering mode (identity for natural)."""
    if mode == "natural":
        return np.arange(mesh.n_cells)
    if mode == "rcm":
        return rcm(mesh)
    if mode == "colour":
        return colour_blocked(mesh)
    if mode == "rcm+colour":
        p1 = rcm(mesh)
        return p1[colour_blocked(M.renumber(mesh, p1))]
    raise ValueError("unknown ordering " + mode)


def apply(mesh: M.Mesh, mode: str) -> M.Mesh:
    if mode == "natural":
        return mesh
    if mode == "rcm":
        return M.renumber(mesh, rcm(mesh))
    if mode == "colour":
        return M.renumber(mesh, colour_blocked(mesh))
    if mode == "rcm+colour":
        return apply(apply(mesh, "rcm"), "colour")
    raise ValueError("unknown ordering " + mode)


def lusgs_levels(mesh: M.Mesh):
    """Forward-sweep level of every cell (reference for the device level build)."""
    lev = np.zeros(mesh.n_cells, np.int64)
    own, nei = mesh.owner, mesh.neighbour
    order = np.argsort(nei, kind="stable")
    # faces sorted by neighbour: level[nei] = max(level[own]) + 1, processed in cell order
    ptr = np.searchsorted(nei[order], np.arange(mesh.n_cells + 1))
    for c in range(mesh.n_cells):
        fs = order[ptr[c]:ptr[c + 1]]
        if len(fs):
            lev[c] = lev[own[fs]].max() + 1
    return lev
