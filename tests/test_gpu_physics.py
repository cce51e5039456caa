"""CUDA path: physics known answers, failure statuses and control logic.

Failures are injected on the host (a NaN written into the uploaded state, an
exactly zero right-hand side); nothing here faults, traps or hangs a GPU.
"""

import numpy as np
import pytest

from icsfoam_gb300 import abi, cases

from test_oracle import exact_riemann  # noqa: E402

pytestmark = pytest.mark.gpu


def open_case(binding, w, **over):
    h = abi.CaseHandle(binding, w.mesh, cases.make_config(binding, w.settings, **over))
    h.set_primitive(w.p, w.U, w.T)
    return h


def test_sod_on_gpu_matches_exact_and_oracle(gpu_binding, oracle_binding):
    w = cases.shock_tube(1000)
    hg = open_case(gpu_binding, w)
    ho = open_case(oracle_binding, w)
    for step in range(100):
        for h in (hg, ho):
            h.begin_time_step()
        while True:
            mg, mo = hg.pseudo_loop(), ho.pseudo_loop()
            assert mg == mo
            if not mg:
                break
            hg.pseudo_iteration()
            ho.pseudo_iteration()
    g, o = hg.get_state(), ho.get_state()
    assert np.abs(g["W"] - o["W"]).max(axis=0).max() / np.abs(o["W"]).max() < 1e-9
    x = w.mesh.C[:, 0]
    ex = exact_riemann(x, 1e-3, (1e5 / (287 * 348.4), 0, 1e5), (1e4 / (287 * 278.7), 0, 1e4))
    assert np.abs(g["W"][:, 0] - ex[:, 0]).mean() < 0.01


@pytest.mark.parametrize("precision", [0, 1])
def test_nonfinite_state_is_reported(gpu_binding, precision):
    w = cases.bump_channel(8, 4, 2, ordering_mode="colour")
    h = open_case(gpu_binding, w, precision=precision)
    W = h.get_state()["W"]
    W[5, 4] = np.nan
    h.set_conservative(W)
    with pytest.raises(abi.IcsError) as e:
        h.residual()
    assert e.value.status == abi.ICS_ERR_NONFINITE
    # the context stays usable: a clean state runs again
    h.set_primitive(w.p, w.U, w.T)
    h.pseudo_iteration()


def still_air(n=6):
    w = cases.shock_tube(n)
    w.p[:] = 1e5
    w.T[:] = 300.0
    w.U[:] = 0.0
    w.settings = dict(w.settings, ddt_scheme=0)
    return w


@pytest.mark.parametrize("lib", ["gpu", "oracle"])
def test_zero_rhs_is_a_krylov_breakdown(gpu_binding, oracle_binding, lib):
    """Still air: the residual is exactly zero, so the first Krylov norm is zero."""
    b = gpu_binding if lib == "gpu" else oracle_binding
    h = open_case(b, still_air())
    src = h.residual()
    assert np.all(src == 0.0)
    h.assemble_jacobian()
    perf, dW, st = h.solve_increment(allow=(abi.ICS_OK, abi.ICS_ERR_BREAKDOWN))
    assert st == abi.ICS_ERR_BREAKDOWN
    assert np.all(dW == 0.0)


def test_pseudo_loop_sequence_matches_oracle(gpu_binding, oracle_binding):
    w = cases.shock_tube(30)
    seqs = []
    for b in (gpu_binding, oracle_binding):
        h = open_case(b, w, n_pseudo_corr=6)
        seq = []
        for _ in range(3):
            h.begin_time_step()
            while h.pseudo_loop():
                h.pseudo_iteration()
                seq.append(1)
            seq.append(0)
        seqs.append(seq)
    assert seqs[0] == seqs[1]


def test_jacobi_preconditioner_parity(gpu_binding, oracle_binding):
    w = cases.bump_channel(10, 4, 3, ordering_mode="colour")
    hs = [open_case(b, w, preconditioner=2) for b in (gpu_binding, oracle_binding)]
    for h in hs:
        h.residual()
        h.assemble_jacobian()
    r = np.random.default_rng(0).standard_normal((w.mesh.n_cells, 5))
    zg, zo = hs[0].precondition(r), hs[1].precondition(r)
    assert np.abs(zg - zo).max() < 1e-11 * np.abs(zo).max()
    pg, dg, _ = hs[0].solve_increment()
    po, do, _ = hs[1].solve_increment()
    assert pg.n_iterations == po.n_iterations
    assert np.abs(dg - do).max() < 1e-9 * np.abs(do).max()


@pytest.mark.parametrize("precision,tol", [(0, 1e-10), (1, 1e-4)])
def test_smooth_solver_parity(gpu_binding, oracle_binding, precision, tol):
    """smoothSolverCoupled (block-Jacobi sweeps) against the oracle."""
    w = cases.bump_channel(10, 4, 3, ordering_mode="colour")
    over = dict(solver=1, n_sweeps=2, max_iter=12, rel_tol=1e-6)
    hg = open_case(gpu_binding, w, precision=precision, **over)
    ho = open_case(oracle_binding, w, **over)
    for h in (hg, ho):
        h.residual()
        h.assemble_jacobian()
    pg, dg, _ = hg.solve_increment()
    po, do, _ = ho.solve_increment()
    assert pg.n_iterations == po.n_iterations
    assert np.abs(dg - do).max() < tol * np.abs(do).max()


def test_profiling_counts_launches(gpu_binding):
    w = cases.bump_channel(8, 4, 2, ordering_mode="colour")
    h = open_case(gpu_binding, w)
    n0 = h.launch_count()
    h.profile(True)
    h.pseudo_iteration()
    h.profile(False)
    prof = h.profile_read()
    n = h.launch_count() - n0
    assert n == sum(v[1] for v in prof.values())
    assert prof["face"][1] == 1 and prof["spmv"][1] >= 2
    assert all(v[0] >= 0 for v in prof.values())


def test_batch_of_independent_cases_equals_sequential_runs(gpu_binding):
    """ics_pseudo_iteration_batch: concurrent handles give bit-identical results."""
    ws = [cases.bump_channel(6 + 2 * k, 4, 2 + k % 2, ordering_mode="colour") for k in range(5)]
    ws.append(cases.shock_tube(50))
    seq = [open_case(gpu_binding, w) for w in ws]
    bat = [open_case(gpu_binding, w) for w in ws]
    for _ in range(4):
        for h in seq:
            h.pseudo_loop()
            h.pseudo_iteration()
        for h in bat:
            h.pseudo_loop()
        stats, status = abi.pseudo_iteration_batch(bat)
        assert status == [abi.ICS_OK] * len(ws)
    for a, b in zip(seq, bat):
        assert np.array_equal(a.get_state()["W"], b.get_state()["W"])
    with pytest.raises(abi.IcsError):
        abi.pseudo_iteration_batch([bat[0], bat[0]])


@pytest.mark.parametrize("unsteady,scalar", [(False, False), (True, True)])
def test_checkpoint_resume_is_bit_exact(gpu_binding, unsteady, scalar):
    """Save after a few iterations, continue; a fresh handle loading the
    checkpoint continues to the identical state."""
    w = cases.bump_channel(24, 8, 4, ordering_mode="colour")
    over = dict(ddt_scheme=2, delta_t=1e-4, n_pseudo_corr=3) if unsteady else {}

    def fresh():
        h = open_case(gpu_binding, w, **over)
        if scalar:
            h.scalar_enable(np.full(w.mesh.n_cells, 0.2), D=0.0, recon=3)
        return h

    def run(h, n):
        for _ in range(n):
            if unsteady and not h.pseudo_loop():
                h.begin_time_step()
            elif not unsteady:
                h.pseudo_loop()
            h.pseudo_iteration()
            if scalar:
                h.scalar_transport(1)

    a = fresh()
    if unsteady:
        a.begin_time_step()
    run(a, 4)
    ck = a.save_checkpoint()
    run(a, 5)
    b = fresh()
    b.load_checkpoint(ck)
    run(b, 5)
    assert np.array_equal(a.get_state()["W"], b.get_state()["W"])
    assert np.array_equal(a.get_boundary_state()["p"], b.get_boundary_state()["p"])
    if scalar:
        assert np.array_equal(a.get_scalar()[0], b.get_scalar()[0])
    other = open_case(gpu_binding, cases.bump_channel(8, 4, 2, ordering_mode="colour"))
    with pytest.raises(abi.IcsError) as e:
        other.load_checkpoint(ck)
    assert e.value.status == abi.ICS_ERR_ARG


def test_bounded_sweep_wait_reports_timeout(gpu_binding):
    """A row left out of a sync-free sweep never writes its result: the rows that
    wait on it give up after a short bound and the status says so; nothing
    faults and the context keeps working."""
    w = cases.bump_channel(24, 8, 4, ordering_mode="natural")
    h = open_case(gpu_binding, w)
    h.residual()
    h.assemble_jacobian()
    assert h.test_sweep_timeout(0, 1000) == abi.ICS_ERR_TIMEOUT  # cell 0 has upper neighbours
    assert h.test_sweep_timeout(w.mesh.n_cells - 1, 1000) == abi.ICS_OK  # nobody depends on the last
    h.pseudo_loop()
    h.pseudo_iteration()
    assert np.all(np.isfinite(h.get_state()["W"]))


def test_precision_change_needs_a_new_jacobian(gpu_binding):
    """The Jacobian's slot storage depends on the precision (25 FP64 entries,
    8 factored FP32 words): switching precision drops the assembled matrix,
    and the re-assembled FP32 one acts like the FP64 one."""
    w = cases.bump_channel(16, 6, 3, ordering_mode="colour")
    h = open_case(gpu_binding, w)
    h.residual()
    h.assemble_jacobian()
    x = np.random.default_rng(3).standard_normal((w.mesh.n_cells, 5))
    y64 = h.matrix_mul(x)
    h.set_config(cases.make_config(gpu_binding, w.settings, precision=1))
    with pytest.raises(abi.IcsError):
        h.matrix_mul(x)
    h.residual()
    h.assemble_jacobian()
    y32 = h.matrix_mul(x)
    scale = np.abs(y64).max(axis=0)
    scale[1:4] = scale[1:4].max()
    assert (np.abs(y32 - y64) / scale).max() < 1e-5


@pytest.mark.parametrize("precision", [0, 1])
def test_gamma_change_needs_a_new_jacobian(gpu_binding, precision):
    """The factored FP32 slots apply gamma when they are used: a new Cp or R
    would mix it with diagonal blocks assembled under the old one, so a change
    of either drops the assembled matrix (in both precisions)."""
    w = cases.bump_channel(16, 6, 3, ordering_mode="colour")
    h = open_case(gpu_binding, w, precision=precision)
    h.residual()
    h.assemble_jacobian()
    x = np.random.default_rng(4).standard_normal((w.mesh.n_cells, 5))
    h.matrix_mul(x)
    h.set_config(cases.make_config(gpu_binding, w.settings, precision=precision, Cp=1040.0))
    with pytest.raises(abi.IcsError):
        h.matrix_mul(x)
    h.residual()
    h.assemble_jacobian()
    assert np.all(np.isfinite(h.matrix_mul(x)))


def test_autotune_keeps_the_results_and_caches_the_choice(gpu_binding):
    """ics_autotune times its launch choices and keeps the fastest; every
    choice gives the same pseudo iterations up to round-off, and a second
    handle of the same shape takes the cached choice."""
    w = cases.bump_channel(48, 16, 16, ordering_mode="colour")
    ref = open_case(gpu_binding, w, precision=1)
    tuned = open_case(gpu_binding, w, precision=1)
    tuned.residual()
    tuned.assemble_jacobian()
    t = tuned.autotune()
    assert t["face_block"] in (64, 128) and t["grad_block"] in (64, 128)
    assert t["mgs_blocks"] in (152, 304, 456, 608) and t["fused_operator"] in (0, 1) and not t["from_cache"]
    assert t["reverse_rows"] in (1, 2)
    for _ in range(3):
        ref.pseudo_loop()
        ref.pseudo_iteration()
        tuned.pseudo_loop()
        tuned.pseudo_iteration()
    Wr, Wt = ref.get_state()["W"], tuned.get_state()["W"]
    scale = np.abs(Wr).max(axis=0)
    assert (np.abs(Wt - Wr) / scale).max() < 1e-6
    other = open_case(gpu_binding, w, precision=1)
    other.residual()
    other.assemble_jacobian()
    t2 = other.autotune()
    assert t2["from_cache"] and {k: t2[k] for k in t2 if k != "from_cache"} == \
        {k: t[k] for k in t if k != "from_cache"}


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("fused", [0, 1])
def test_reverse_rows_per_thread_keep_every_bit(gpu_binding, precision, fused):
    """ics_set_tuning(reverse_rows=2): two rows of a reverse LU-SGS level per
    thread, each with the one-row arithmetic: the preconditioner and three
    pseudo iterations are bit-identical to one row per thread, on the two-level
    (colour-blocked) schedule of 4320 rows (level launches, not the one-CTA
    walk), with and without the fused operator."""
    for order in ("colour",):
        w = cases.bump_channel(40, 12, 9, ordering_mode=order)
        hs = [open_case(gpu_binding, w, precision=precision) for _ in range(2)]
        for h, rows in zip(hs, (1, 2)):
            h.set_tuning(fused_operator=fused, reverse_rows=rows)
            h.residual()
            h.assemble_jacobian()
        r = np.random.default_rng(5).standard_normal((w.mesh.n_cells, 5))
        assert np.array_equal(hs[0].precondition(r), hs[1].precondition(r)), order
        for _ in range(3):
            for h in hs:
                h.pseudo_loop()
                h.pseudo_iteration()
        assert np.array_equal(hs[0].get_state()["W"], hs[1].get_state()["W"]), order
    with pytest.raises(abi.IcsError):
        hs[0].set_tuning(reverse_rows=3)
