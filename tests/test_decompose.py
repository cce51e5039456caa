"""Domain decomposition across ranks on two gloo ranks (CPU, the oracle per rank).

The partitioned case must reproduce the single-domain one: each rank's
owned rows of the residual source and of the Jacobian action (after halo
exchanges of the state and of the vector) equal the single-domain rows to
1e-12 of each equation's max-norm; the LU-SGS of each rank over its own
internal faces equals the single-domain LU-SGS with the faces between the
ranks removed (block-Jacobi across ranks, as the reference's lusgs.C does
across processor patches); and a GMRES whose dot products are all-reduced
over the ranks solves the single-domain system.  The numpy LU-SGS used for
the block-Jacobi comparison is first pinned to the oracle's LU-SGS on the
undivided mesh.
"""

import os
import socket

import numpy as np
import pytest

from icsfoam_gb300 import abi, cases
from icsfoam_gb300 import decompose as D

from test_gpu_parity import perturb, relerr  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _workload():
    return perturb(cases.bump_channel(24, 8, 4, ordering_mode="natural"))


def _global(binding, w):
    h = abi.CaseHandle(binding, w.mesh, cases.make_config(binding, w.settings))
    h.set_primitive(w.p, w.U, w.T)
    return h


def _gmres(A, M, dots, b, tol=1e-11, m=30, cycles=40):
    """Right-preconditioned restarted GMRES on owned rows; dots(w, [v...])
    returns the global dot products (one all-reduce per call)."""
    x = np.zeros_like(b)
    bn = np.sqrt(dots(b, [b])[0])
    r = b.copy()
    for _ in range(cycles):
        beta = np.sqrt(dots(r, [r])[0])
        if beta <= tol * bn:
            break
        V = [r / beta]
        H = np.zeros((m + 1, m))
        for i in range(m):
            w = A(M(V[i]))
            h1 = dots(w, V)
            w = w - sum(c * v for c, v in zip(h1, V))
            h2 = dots(w, V)
            w = w - sum(c * v for c, v in zip(h2, V))
            H[: i + 1, i] = h1 + h2
            H[i + 1, i] = np.sqrt(dots(w, [w])[0])
            V.append(w / H[i + 1, i])
        e = np.zeros(m + 1)
        e[0] = beta
        y = np.linalg.lstsq(H, e, rcond=None)[0]
        x = x + M(sum(c * v for c, v in zip(y, V[:m])))
        r = b - A(x)
    return x


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch.distributed as dist

    import oracle

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ob = oracle.binding()
        w = _workload()
        part = D.partition(w.mesh, world)
        subs = D.decompose(w.mesh, part)
        plans = D.halo_plans(subs, part)
        sub = subs[rank]
        h = abi.CaseHandle(ob, sub.mesh, cases.make_config(ob, w.settings))
        h.set_primitive(w.p[sub.cells], w.U[sub.cells], w.T[sub.cells])
        ds = D.DistributedSystem(sub, plans[rank], h, dist)
        # the state of the owned cells, the halo filled by the exchange
        ds.set_state(h.get_state()["W"][: sub.n_owned])
        res = ds.residual()
        ds.assemble_jacobian()
        x = np.random.default_rng(1).standard_normal((w.mesh.n_cells, 5))
        y = ds.matrix_mul(x[sub.owned])
        z = ds.lusgs(x[sub.owned])
        b = res.copy()
        sol = _gmres(ds.matrix_mul, ds.lusgs, lambda a, vs: ds.dots(a, vs), b)
        out[rank] = {"owned": sub.owned, "res": res, "y": y, "z": z, "sol": sol, "n_halo1": sub.n_halo1,
                     "n_local": sub.mesh.n_cells}
    finally:
        dist.destroy_process_group()


def test_numpy_lusgs_matches_the_oracle(oracle_binding):
    w = _workload()
    h = _global(oracle_binding, w)
    h.residual()
    h.assemble_jacobian()
    Dg, Lg, Ug = h.get_jacobian()
    r = np.random.default_rng(2).standard_normal((w.mesh.n_cells, 5))
    got = D.lusgs_ldu(w.mesh.n_cells, w.mesh.owner, w.mesh.neighbour, Dg, Lg, Ug, r)
    assert relerr(got, h.precondition(r)) < 1e-12


def test_partition_and_halo_plans():
    w = _workload()
    part = D.partition(w.mesh, 3)
    assert np.bincount(part).max() - np.bincount(part).min() <= 1
    subs = D.decompose(w.mesh, part)
    plans = D.halo_plans(subs, part)
    for s in subs:
        assert np.all(part[s.owned] == s.rank) and np.all(part[s.halo] != s.rank)
        assert np.all(s.mesh.owner < s.mesh.neighbour)
        # every neighbour of an owned cell is local (two layers reach the second ring)
        loc = set(s.cells.tolist())
        for o, n in zip(w.mesh.owner, w.mesh.neighbour):
            if part[o] == s.rank:
                assert int(n) in loc
            if part[n] == s.rank:
                assert int(o) in loc
        for q, idx in plans[s.rank].recv.items():
            assert np.array_equal(subs[q].owned[plans[q].send[s.rank]], s.cells[idx])


def test_two_rank_residual_matvec_block_jacobi_and_gmres(oracle_binding):
    pytest.importorskip("torch")
    import torch.multiprocessing as mp

    w = _workload()
    h = _global(oracle_binding, w)
    res = h.residual()
    h.assemble_jacobian()
    Dg, Lg, Ug = h.get_jacobian()
    x = np.random.default_rng(1).standard_normal((w.mesh.n_cells, 5))
    y = h.matrix_mul(x)
    part = D.partition(w.mesh, 2)
    # the single-domain LU-SGS without the faces between the two parts
    keep = part[w.mesh.owner] == part[w.mesh.neighbour]
    z = D.lusgs_ldu(w.mesh.n_cells, w.mesh.owner[keep], w.mesh.neighbour[keep], Dg, Lg[keep], Ug[keep], x)
    port = _free_port()
    mgr = mp.Manager()
    out = mgr.dict()
    mp.spawn(_worker, args=(2, port, out), nprocs=2, join=True)
    got_res, got_y, got_z, got_sol = (np.zeros_like(x) for _ in range(4))
    for r in range(2):
        o = out[r]
        assert o["n_halo1"] > 0 and o["n_local"] > len(o["owned"])
        got_res[o["owned"]] = o["res"]
        got_y[o["owned"]] = o["y"]
        got_z[o["owned"]] = o["z"]
        got_sol[o["owned"]] = o["sol"]
    assert relerr(got_res, res) < 1e-12
    assert relerr(got_y, y) < 1e-12
    assert relerr(got_z, z) < 1e-12
    # the distributed solve of A x = R V agrees with the single-domain matrix
    assert relerr(h.matrix_mul(got_sol), res) < 1e-9
