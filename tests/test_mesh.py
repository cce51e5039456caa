"""Mesh generation, geometry and orderings (host side, CPU only)."""

from collections import deque

import numpy as np
import pytest

from icsfoam_gb300 import cases, mesh as M, ordering


def closure(m):
    acc = np.zeros((m.n_cells, 3))
    np.add.at(acc, m.owner, m.Sf)
    np.add.at(acc, m.neighbour, -m.Sf)
    np.add.at(acc, m.b_cell, m.b_Sf)
    return np.abs(acc).max()


@pytest.mark.parametrize("build", [
    lambda: cases.bump_channel(16, 6, 4, ordering_mode="natural"),
    lambda: cases.bump_channel(16, 6, 4, ordering_mode="colour"),
    lambda: cases.random_box(5),
])
def test_geometry_invariants(build):
    m = build().mesh
    assert np.all(m.owner < m.neighbour)
    key = m.owner.astype(np.int64) * m.n_cells + m.neighbour
    assert np.all(np.diff(key) > 0), "internal faces must be upper-triangular"
    assert closure(m) < 1e-12 * np.abs(m.Sf).max()
    assert np.all(m.V > 0)
    assert np.all((m.weights > 0) & (m.weights < 1))
    assert np.all(m.nonorth_delta_coeffs > 0) and np.all(m.b_delta_coeffs > 0)


def test_box_volume_and_centres():
    w = cases.random_box(4)
    m = w.mesh
    assert abs(m.V.sum() - 1.0) < 1e-12   # displaced vertices keep the box volume
    assert np.all((m.C > 0) & (m.C < 1))


def test_shock_tube_topology():
    m = cases.shock_tube(50).mesh
    assert (m.n_cells, m.n_faces, m.n_bfaces) == (50, 49, 2)
    assert m.solution_d == (1, -1, -1)
    assert np.allclose(m.V, 0.2 ** 3)


# ------------------------------------------------------------------ orderings
def py_greedy_colour(n, own, nei):
    adj = [[] for _ in range(n)]
    for o, q in zip(own, nei):
        adj[o].append(q)
        adj[q].append(o)
    col = [-1] * n
    for i in range(n):
        used = {col[j] for j in adj[i] if col[j] >= 0}
        c = 0
        while c in used:
            c += 1
        col[i] = c
    return np.array(col)


def py_rcm(n, own, nei):
    """Independent restatement of the documented RCM tie-break."""
    adj = [set() for _ in range(n)]
    for o, q in zip(own, nei):
        adj[o].add(q)
        adj[q].add(o)
    deg = [len(a) for a in adj]
    placed = [False] * n
    order = []

    def levels(root):
        lev = {root: 0}
        dq = deque([root])
        while dq:
            u = dq.popleft()
            for v in sorted(adj[u]):
                if v not in lev:
                    lev[v] = lev[u] + 1
                    dq.append(v)
        d = max(lev.values())
        return d, [v for v, l in lev.items() if l == d]

    for seed in range(n):
        if placed[seed]:
            continue
        comp, dq, seen = [], deque([seed]), {seed}
        while dq:
            u = dq.popleft()
            comp.append(u)
            for v in adj[u]:
                if v not in seen:
                    seen.add(v)
                    dq.append(v)
        root = min(comp, key=lambda v: (deg[v], v))
        depth, last = levels(root)
        while True:
            cand = min(last, key=lambda v: (deg[v], v))
            d2, last2 = levels(cand)
            if d2 > depth:
                depth, root, last = d2, cand, last2
            else:
                break
        start = len(order)
        order.append(root)
        placed[root] = True
        h = start
        while h < len(order):
            u = order[h]
            h += 1
            for v in sorted((v for v in adj[u] if not placed[v]), key=lambda v: (deg[v], v)):
                placed[v] = True
                order.append(v)
    return np.array(order[::-1])


@pytest.mark.parametrize("build", [lambda: cases.bump_channel(12, 5, 3, ordering_mode="natural"),
                                   lambda: cases.random_box(5, ordering_mode="natural")])
def test_colouring_bit_exact_and_valid(build):
    m = build().mesh
    col, ncol = ordering.greedy_colour(m)
    ref = py_greedy_colour(m.n_cells, m.owner, m.neighbour)
    assert np.array_equal(col, ref)
    assert ncol == col.max() + 1
    assert np.all(col[m.owner] != col[m.neighbour]), "no two neighbours share a colour"


@pytest.mark.parametrize("build", [lambda: cases.bump_channel(12, 5, 3, ordering_mode="natural"),
                                   lambda: cases.random_box(5, ordering_mode="natural")])
def test_rcm_bit_exact(build):
    m = build().mesh
    assert np.array_equal(ordering.rcm(m), py_rcm(m.n_cells, m.owner, m.neighbour))


def test_rcm_reduces_bandwidth():
    m = cases.random_box(6, ordering_mode="natural").mesh  # randomly permuted cells
    bw0 = np.abs(m.owner.astype(int) - m.neighbour).max()
    m2 = ordering.apply(m, "rcm")
    bw1 = np.abs(m2.owner.astype(int) - m2.neighbour).max()
    assert bw1 < bw0 / 2


def test_lusgs_levels():
    nx, ny, nz = 8, 5, 3
    m = cases.bump_channel(nx, ny, nz, ordering_mode="natural").mesh
    assert ordering.lusgs_levels(m).max() + 1 == nx + ny + nz - 2
    mc = ordering.apply(m, "colour")
    _, ncol = ordering.greedy_colour(m)
    assert ncol == 2
    assert ordering.lusgs_levels(mc).max() + 1 == ncol


def test_renumber_preserves_geometry():
    m = cases.bump_channel(10, 4, 3, ordering_mode="natural").mesh
    perm = np.random.default_rng(0).permutation(m.n_cells)
    m2 = M.renumber(m, perm)
    assert np.allclose(np.sort(m2.V), np.sort(m.V))
    assert np.allclose(m2.V, m.V[perm])
    assert np.allclose(m2.C, m.C[perm])
    assert abs(np.abs(m2.Sf).sum() - np.abs(m.Sf).sum()) < 1e-12
