"""Domain decomposition of a case across ranks (one GPU per rank).

The reference runs in parallel by OpenFOAM domain decomposition: every MPI
rank owns a subdomain of cells, processor patches exchange the neighbour
values of every field and of every Krylov vector (blockFvMatrix.C:355-592,
blockFvMatrixUpdateMatrixInterfaces.C:105-185), each GMRES dot product and
norm is one global sum (gmres.C:936-1011), and LU-SGS sweeps only the
rank's internal faces, i.e. it is block-Jacobi across ranks
(lusgs.C:147-150, 181).  This module is that decomposition for handles of
the C ABI, one handle per rank:

* ``partition``  cells into ``n`` parts by a geometric split along x, the
  decomposePar "simple" layout (equal cell counts, cells ordered by centre);
* ``decompose``  each part's local mesh: its owned cells (numbered first,
  in global order) and two layers of halo cells, with every internal face
  among them and their boundary faces; the halo's outer faces become a
  zeroGradient patch.  Two layers make the owned rows exact: the face
  fluxes of an owned cell need the limited gradients of its neighbours,
  whose Gauss gradients and cellLimited bounds read the second layer;
* ``HaloPlan``   who sends which owned cells to whom, and where they land;
* ``DistributedSystem`` the pieces of a distributed pseudo iteration on top
  of per-rank handles and ``torch.distributed`` (gloo on CPU, NCCL across
  GPUs): residual and Jacobian rows of the owned cells after a halo
  exchange of the state, the matrix action with a halo exchange of the
  vector, global dot products (one all-reduce of all the Gram-Schmidt dots
  of a Krylov step), and the block-Jacobi LU-SGS of the reference across
  ranks.

Meshes with cyclic patches are not decomposed here.
"""

from __future__ import annotations

import dataclasses
from typing import Dict, List

import numpy as np

from . import mesh as M

HALO_PATCH = "procBoundary"


def partition(mesh: M.Mesh, n_parts: int) -> np.ndarray:
    """Part of every cell: equal-count slabs of the cells ordered by (x, y, z)."""
    if n_parts < 1:
        raise ValueError("n_parts must be >= 1")
    order = np.lexsort((mesh.C[:, 2], mesh.C[:, 1], mesh.C[:, 0]))
    part = np.empty(mesh.n_cells, np.int32)
    for p, chunk in enumerate(np.array_split(order, n_parts)):
        part[chunk] = p
    return part


def _neighbours(mesh: M.Mesh, cells: np.ndarray) -> np.ndarray:
    """Cells sharing an internal face with any of ``cells``."""
    sel = np.zeros(mesh.n_cells, bool)
    sel[cells] = True
    own, nei = mesh.owner, mesh.neighbour
    a = nei[sel[own]]
    b = own[sel[nei]]
    return np.unique(np.concatenate([a, b]))


@dataclasses.dataclass
class Subdomain:
    rank: int
    cells: np.ndarray        # global id of every local cell: owned (first), then the halo
    n_owned: int
    n_halo1: int             # first-layer halo cells (after the owned ones)
    mesh: M.Mesh             # local mesh in OpenFOAM LDU order
    local_of: Dict[int, int] = dataclasses.field(default_factory=dict, repr=False)

    @property
    def owned(self) -> np.ndarray:
        return self.cells[: self.n_owned]

    @property
    def halo(self) -> np.ndarray:
        return self.cells[self.n_owned:]


def decompose(mesh: M.Mesh, part: np.ndarray, layers: int = 2) -> List[Subdomain]:
    if mesh.b_partner is not None and np.any(mesh.b_partner >= 0):
        raise ValueError("meshes with cyclic patches are not decomposed")
    n_parts = int(part.max()) + 1
    subs = []
    for p in range(n_parts):
        owned = np.nonzero(part == p)[0]
        have = np.zeros(mesh.n_cells, bool)
        have[owned] = True
        rings = []
        frontier = owned
        for _ in range(layers):
            nb = _neighbours(mesh, frontier)
            nb = nb[~have[nb]]
            have[nb] = True
            rings.append(nb)
            frontier = nb
        cells = np.concatenate([owned] + rings).astype(np.int64)
        subs.append(_local_mesh(mesh, p, cells, len(owned), len(rings[0]) if rings else 0))
    return subs


def _local_mesh(mesh: M.Mesh, rank: int, cells: np.ndarray, n_owned: int, n_halo1: int) -> Subdomain:
    N = mesh.n_cells
    loc = np.full(N, -1, np.int64)
    loc[cells] = np.arange(len(cells))
    own_g, nei_g = mesh.owner.astype(np.int64), mesh.neighbour.astype(np.int64)
    lo, ln = loc[own_g], loc[nei_g]
    inner = (lo >= 0) & (ln >= 0)
    # internal faces among the local cells, re-oriented so that owner < neighbour locally
    fi = np.nonzero(inner)[0]
    a, b = lo[fi], ln[fi]
    flip = a > b
    o2 = np.where(flip, b, a)
    n2 = np.where(flip, a, b)
    sgn = np.where(flip, -1.0, 1.0)[:, None]
    Sf = mesh.Sf[fi] * sgn
    w = np.where(flip, 1.0 - mesh.weights[fi], mesh.weights[fi])
    order = np.lexsort((n2, o2))
    fi, o2, n2, Sf, w = fi[order], o2[order], n2[order], Sf[order], w[order]
    # faces from the outer halo layer to cells outside: a zeroGradient patch
    cut = np.nonzero((lo >= 0) ^ (ln >= 0))[0]
    cut_cell = np.where(lo[cut] >= 0, lo[cut], ln[cut])
    cut_out = np.where(lo[cut] >= 0, 1.0, -1.0)[:, None]  # area vector pointing out of the local cell
    cut_Sf = mesh.Sf[cut] * cut_out
    cut_Cf = mesh.Cf[cut]
    cut_dc = 2.0 * mesh.delta_coeffs[cut]
    # the original boundary faces of the local cells, patch by patch
    bsel = loc[mesh.b_cell.astype(np.int64)] >= 0
    patches = list(mesh.patches)
    b_cell = loc[mesh.b_cell[bsel].astype(np.int64)]
    b_patch = mesh.b_patch[bsel].astype(np.int64)
    b_Sf, b_Cf, b_dc = mesh.b_Sf[bsel], mesh.b_Cf[bsel], mesh.b_delta_coeffs[bsel]
    if len(cut):
        patches = patches + [M.Patch(HALO_PATCH, M.PATCH_ZERO_GRADIENT)]
        b_cell = np.concatenate([b_cell, cut_cell])
        b_patch = np.concatenate([b_patch, np.full(len(cut), len(patches) - 1)])
        b_Sf = np.concatenate([b_Sf, cut_Sf])
        b_Cf = np.concatenate([b_Cf, cut_Cf])
        b_dc = np.concatenate([b_dc, cut_dc])
    bo = np.argsort(b_patch, kind="stable")
    lm = M.Mesh(
        n_cells=len(cells),
        owner=o2.astype(np.int32), neighbour=n2.astype(np.int32),
        Sf=np.ascontiguousarray(Sf), Cf=np.ascontiguousarray(mesh.Cf[fi]),
        weights=np.ascontiguousarray(w), delta_coeffs=mesh.delta_coeffs[fi].copy(),
        nonorth_delta_coeffs=mesh.nonorth_delta_coeffs[fi].copy(),
        C=np.ascontiguousarray(mesh.C[cells]), V=mesh.V[cells].copy(),
        b_cell=b_cell[bo].astype(np.int32), b_Sf=np.ascontiguousarray(b_Sf[bo]),
        b_Cf=np.ascontiguousarray(b_Cf[bo]), b_delta_coeffs=np.ascontiguousarray(b_dc[bo]),
        b_patch=b_patch[bo].astype(np.int32), patches=patches, solution_d=mesh.solution_d,
    )
    return Subdomain(rank, cells, n_owned, n_halo1, lm)


@dataclasses.dataclass
class HaloPlan:
    """send[q]: local indices of this rank's owned cells that rank q holds as
    halo; recv[q]: local indices of this rank's halo cells owned by rank q, in
    the order q sends them."""
    send: Dict[int, np.ndarray]
    recv: Dict[int, np.ndarray]


def halo_plans(subs: List[Subdomain], part: np.ndarray) -> List[HaloPlan]:
    plans = [HaloPlan({}, {}) for _ in subs]
    for s in subs:
        halo = s.halo
        owner_rank = part[halo]
        for q in np.unique(owner_rank):
            q = int(q)
            glob = halo[owner_rank == q]                       # increasing global ids
            plans[s.rank].recv[q] = s.n_owned + np.nonzero(owner_rank == q)[0]
            oq = subs[q]
            pos = np.searchsorted(oq.owned, glob)              # owned cells are in global order
            plans[q].send[s.rank] = pos
    return plans


class DistributedSystem:
    """The distributed pieces of a pseudo iteration on one rank.

    ``handle`` is this rank's CaseHandle on ``sub.mesh`` (oracle or CUDA
    library); ``dist`` is ``torch.distributed`` with an initialised process
    group.  Vectors passed in and out are the rank's owned rows [n_owned][5].
    """

    def __init__(self, sub: Subdomain, plan: HaloPlan, handle, dist):
        self.sub, self.plan, self.h, self.dist = sub, plan, handle, dist
        self.rank = dist.get_rank()

    # -------------------------------------------------------------- exchange
    def exchange(self, local: np.ndarray) -> np.ndarray:
        """Fill the halo rows of ``local`` ([n_local][k]) from their owners."""
        import torch

        reqs, bufs = [], []
        for q, idx in sorted(self.plan.send.items()):
            t = torch.from_numpy(np.ascontiguousarray(local[idx]))
            reqs.append(self.dist.isend(t, q))
            bufs.append(t)
        recv = {}
        for q, idx in sorted(self.plan.recv.items()):
            t = torch.empty((len(idx),) + local.shape[1:], dtype=torch.float64)
            reqs.append(self.dist.irecv(t, q))
            recv[q] = t
        for r in reqs:
            r.wait()
        for q, t in recv.items():
            local[self.plan.recv[q]] = t.numpy()
        return local

    def _extend(self, owned: np.ndarray) -> np.ndarray:
        out = np.zeros((self.sub.mesh.n_cells,) + owned.shape[1:])
        out[: self.sub.n_owned] = owned
        return self.exchange(out)

    # -------------------------------------------------------------- reductions
    def allreduce(self, values: np.ndarray) -> np.ndarray:
        """Global sums of a vector of partial sums: one all-reduce for all of
        them (all the Gram-Schmidt dots of a Krylov step go in one call)."""
        import torch

        t = torch.from_numpy(np.ascontiguousarray(values, np.float64))
        self.dist.all_reduce(t)
        return t.numpy()

    def dots(self, w: np.ndarray, vs: List[np.ndarray]) -> np.ndarray:
        return self.allreduce(np.array([float(np.sum(w * v)) for v in vs]))

    # -------------------------------------------------------------- operators
    def set_state(self, W_owned: np.ndarray):
        """The conservative state of the owned cells; halo cells from their owners."""
        self.h.set_conservative(self._extend(W_owned))

    def residual(self) -> np.ndarray:
        return self.h.residual()[: self.sub.n_owned]

    def assemble_jacobian(self):
        self.h.assemble_jacobian()
        D, L, U = self.h.get_jacobian()
        self.D, self.L, self.U = D, L, U

    def matrix_mul(self, x_owned: np.ndarray) -> np.ndarray:
        """Rows of A x for the owned cells; the halo's x comes from its owners."""
        return self.h.matrix_mul(self._extend(x_owned))[: self.sub.n_owned]

    def lusgs(self, r_owned: np.ndarray) -> np.ndarray:
        """The reference's LU-SGS over this rank's internal faces only
        (block-Jacobi across ranks, lusgs.C:147-150)."""
        m = self.sub.mesh
        n = self.sub.n_owned
        keep = (m.owner < n) & (m.neighbour < n)
        return lusgs_ldu(n, m.owner[keep], m.neighbour[keep], self.D[:n], self.L[keep], self.U[keep], r_owned)


def lusgs_ldu(n: int, owner: np.ndarray, neighbour: np.ndarray, D: np.ndarray, L: np.ndarray, U: np.ndarray,
              r: np.ndarray) -> np.ndarray:
    """LU-SGS with the reference's scalar diagonal on LDU blocks (lusgs.C):
    rD = 1 / max |diagonal entries| of each cell's block; forward sweep in
    cell order, delta*_c = rD_c (r_c - sum over lower neighbours l of
    lower_f delta*_l); reverse sweep, delta_c = delta*_c - rD_c sum over upper
    neighbours u of upper_f delta_u.  Faces are the rank's internal faces."""
    rD = 1.0 / np.max(np.abs(np.einsum("cii->ci", D)), axis=1)
    lower_of = [[] for _ in range(n)]
    upper_of = [[] for _ in range(n)]
    for f, (o, nb) in enumerate(zip(owner, neighbour)):
        lower_of[nb].append((f, o))   # row nb, column o < nb: lower block of face f
        upper_of[o].append((f, nb))   # row o, column nb > o: upper block of face f
    d = np.array(r, dtype=np.float64, copy=True)
    for c in range(n):
        acc = d[c].copy()
        for f, o in lower_of[c]:
            acc -= L[f] @ d[o]
        d[c] = rD[c] * acc
    for c in range(n - 1, -1, -1):
        acc = np.zeros(5)
        for f, nb in upper_of[c]:
            acc += U[f] @ d[nb]
        d[c] = d[c] - rD[c] * acc
    return d
