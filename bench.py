#!/usr/bin/env python
"""Benchmark of the implicit coupled pseudo-time iteration on one GB300.

Workload: inviscid transonic bump channel, 256x64x64 hex cells (1,048,576),
HLLC with MUSCL / Venkatakrishnan reconstruction, steady local time stepping
with the SER CFL ramp 1 -> 200, GMRES(8) + LU-SGS on the colour-blocked cell
numbering.  Synthetic mesh and uniform initial state (generated, seeded).

A step is one pseudo-time (Newton) iteration: residual, local time step,
Jacobian assembly, GMRES solve, state update.  ``value`` is cell-iterations
per second of the mixed-precision path (FP64 residual and update, FP32
Jacobian, preconditioner and Krylov basis) with all state resident in HBM;
the FP64 path is timed the same way beside it.  The working set (state,
Jacobian, Krylov basis: several GB) is far larger than the 129 MB L2, so no
L2 flush is needed between steps.

Other legs in the JSON line: iterations and seconds to a 1e-8 drop of the
density residual (mixed and FP64), the end-to-end rate through the C ABI with
host buffers, the roofline of the dominant kernel, SM clocks sampled during
the timed region, and the CPU oracle timed on a bounded sample.

``--impl reference`` times the CPU oracle (the reference algorithm restated
in C++) on 64x16x16 samples of the same workload, one process per host core.
"""

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "cell-iters/s to 1e-8 residual drop, mixed vs FP64 on GB300; flux+SpMV HBM GB/s"
UNIT = "cell-iters/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--nx", type=int, default=256)
    ap.add_argument("--ny", type=int, default=64)
    ap.add_argument("--nz", type=int, default=64)
    ap.add_argument("--to-solution", type=int, default=1, help="also run to the 1e-8 drop")
    ap.add_argument("--solution-cap-s", type=float, default=60.0,
                    help="time cap of the mixed-precision leg to 1e-8 (the FP64 leg gets 2.5x)")
    ap.add_argument("--plateau-cap-s", type=float, default=15.0,
                    help="seconds of the configured Venkatakrishnan limiter (mixed) recording its plateau")
    ap.add_argument("--study-box-first", type=int, default=0,
                    help="with --convergence-study: only the viscous box of this size, first order")
    ap.add_argument("--batch", type=int, default=0,
                    help="only the batch of this many independent shock-tube cases")
    ap.add_argument("--batch-stacked-only", type=int, default=0,
                    help="with --batch: only the cases stacked in one handle")
    ap.add_argument("--adjoint", type=int, default=0,
                    help="only the reverse-mode VJP and the adjoint solve on the 240x128x128 swept bump")
    ap.add_argument("--convergence-study", type=int, default=0,
                    help="only record the GPU and oracle rho residual histories of the reduced workloads")
    ap.add_argument("--viscous-solution", type=int, default=0,
                    help="only run the 200^3 viscous box (8M cells) to --viscous-target in both precisions")
    ap.add_argument("--viscous-target", type=float, default=1e-8,
                    help="rho residual drop (from the peak) the viscous box is run to")
    ap.add_argument("--autotune", type=int, default=1,
                    help="ics_autotune the headline handles after warm-up (launch shapes only)")
    ap.add_argument("--e2e-steps", type=int, default=10)
    ap.add_argument("--cpu-seconds", type=float, default=15.0,
                    help="timed seconds of the CPU baseline (at least one full-mesh iteration per core)")
    ap.add_argument("--profile", type=int, default=1, help="per-kernel CUDA events in the timed region")
    ap.add_argument("--extras", type=int, default=1,
                    help="also time the Harmonic Balance sweep, the batch of independent cases and the "
                         "residual derivatives")
    return ap.parse_args()


# ------------------------------------------------------------------ ranks
class Dist:
    def __init__(self, n):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as td

            td.init_process_group("gloo")
            self.td = td
            self.pg = True

    def barrier(self):
        if self.pg:
            self.td.barrier()

    def max(self, v):
        if not self.pg:
            return v
        import torch

        t = torch.tensor([v], dtype=torch.float64)
        self.td.all_reduce(t, op=self.td.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.pg:
            self.td.destroy_process_group()


# ------------------------------------------------------------------ clocks
class ClockSampler:
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.rows = []
        self.p = None
        self.index = index

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.p = None

    def _read(self):
        for line in self.p.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 8:
                self.rows.append(parts)

    def stop(self):
        if self.p:
            self.p.terminate()
            try:
                self.p.wait(5)
            except subprocess.TimeoutExpired:
                self.p.kill()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        sm, mx, reasons = [], [], set()
        for r in self.rows:
            try:
                sm.append(float(r[0]))
                mx.append(float(r[1]))
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if r[4 + k].lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------- algorithmic bytes
def kernel_bytes(kind, N, F, B, nslots, mixed, nlev):
    """Compulsory DRAM bytes of one launch of a kernel class (each array once).

    Off-diagonal slots hold ow words: 8 in FP32 storage (the factored block:
    scaled normal, side velocity and energy, identity multiple), 25 in FP64;
    diagonal blocks hold 25.
    """
    pb = 4 if mixed else 8   # block entries
    pv = 4 if mixed else 8   # Krylov vectors
    ow = 8 if mixed else 25  # words per off-diagonal slot
    if kind == "face":       # MUSCL face flux: gathered cell fields + face geometry + outputs
        return 264 * N + 232 * F
    if kind == "grad":
        return 268 * N + 96 * F
    if kind == "cellres":
        return 136 * N + 64 * F
    if kind == "jac_rows":
        return (112 + 2 * ow * pb) * F + (25 * pb + 16 + pb) * N
    if kind == "spmv":
        return 25 * pb * N + 2 * ow * pb * F + 8 * F + 10 * pv * N
    if kind in ("lusgs_fwd", "lusgs_rev"):
        # colour-blocked 2-level schedule: one launch per sweep (forward level 0 has no lower
        # neighbours; the last forward level is fused with the first reverse one), reading all F
        # slots of its triangle, rD and r of its N/2 rows, the neighbours' deltas, writing deltas
        return ow * pb * F + pb * N / 2 + 3 * 5 * pv * N / 2 + 4 * F
    if kind == "op0":   # fused operator, pass 1: (A x) on the level-0 half of the rows
        return 25 * pb * N / 2 + ow * pb * F + 5 * pv * N + 5 * pv * N / 2 + 4 * F
    if kind == "op1":   # pass 2: (A x) + forward sweep + first reverse on the other half
        return 25 * pb * N / 2 + ow * pb * F + 10 * pv * N + pb * N + 4 * F
    if kind == "mgs":
        return 20 * pv * N
    return None


# What bounds each kernel class: the FP64 pipe (GB300 runs FP64 at ~1.3
# TFLOP/s) or HBM.  The residual's face and gradient kernels and the
# dual-number / reverse-mode derivative kernels are FP64-ALU bound in both
# precisions; the Jacobian row assembly is FP64-ALU bound when it writes
# FP64 blocks; the Krylov passes are HBM bound.
FP64_BOUND = {"face", "grad", "bface", "tangent", "adjoint", "exact"}


def kernel_bound(kind, mixed):
    if kind in FP64_BOUND or (kind == "jac_rows" and not mixed):
        return "fp64"
    return "hbm"


# FP64 flops of one unit of work (a face for "face", a cell for "grad"),
# HLLC + MUSCL / cellLimited<Venkatakrishnan>: counted by ncu from the
# executed DFMA (2 flops), DADD and DMUL instructions of one launch
# (profiles/fp64_face_grad_bump_128x64x64.md), divided by the faces / cells
FP64_FLOPS_PER_UNIT = {"face": 319.8, "grad": 1013.2}


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def load_traffic():
    """Per-launch DRAM bytes of kernel classes from the committed ncu summary."""
    p = os.path.join(ROOT, "profiles", "ncu_dram_traffic.txt")
    out = {}
    try:
        with open(p) as f:
            for line in f:
                if line.startswith("#") or not line.strip():
                    continue
                kind, cells, prec, byts = line.split()[:4]
                out[(kind, prec)] = (int(cells), float(byts))
    except OSError:
        pass
    return out


# ------------------------------------------------------------------ legs
# launch choices picked by ics_autotune on the headline workload (per
# precision), applied to the later handles of the same mesh
TUNING = {}
TUNE_KEYS = ("face_block", "grad_block", "mgs_blocks", "fused_operator", "reverse_rows")


def tuned(h, prec):
    if prec in TUNING:
        h.set_tuning(**TUNING[prec])
    return h


def run_timed(w, prec, steps, warmup, dist, profile, autotune=True):
    from icsfoam_gb300 import cases, gpu

    b = gpu.binding()
    h = gpu.open_case(w.mesh, cases.make_config(b, w.settings, precision=prec))
    h.set_primitive(w.p, w.U, w.T)
    fp64_rate = h.measure_fp64_rate()
    for _ in range(warmup):
        h.pseudo_loop()
        h.pseudo_iteration()
    if autotune:
        # ics_autotune on the warmed-up state (outside the timed region)
        t = h.autotune()
        TUNING[prec] = {k: t[k] for k in TUNE_KEYS}
    clocks = ClockSampler(0)
    clocks.start()
    dist.barrier()
    l0 = h.launch_count()
    h.timer_start()
    last = None
    cycles = 0
    for _ in range(steps):
        h.pseudo_loop()
        last = h.pseudo_iteration()
        cycles += last.perf.n_iterations
    ms = h.timer_stop()
    launches = h.launch_count() - l0
    ck = clocks.stop()
    ms = dist.max(ms)
    h.close()
    kern = None
    if profile:
        # replay the same iterations on a fresh handle with a CUDA event pair
        # around every launch on the handle's stream: per-kernel-class device
        # time of exactly the timed work (direct launches instead of the
        # captured GMRES cycle graph)
        h = tuned(gpu.open_case(w.mesh, cases.make_config(b, w.settings, precision=prec)), prec)
        h.set_primitive(w.p, w.U, w.T)
        for _ in range(warmup):
            h.pseudo_loop()
            h.pseudo_iteration()
        h.profile(True)
        for _ in range(steps):
            h.pseudo_loop()
            h.pseudo_iteration()
        h.profile(False)
        kern = h.profile_read()
        h.close()
    return {"ms": ms, "launches": launches, "kernels": kern, "clocks": ck,
            "last_rho_l2": last.rho_l2_residual if last else None, "fp64_rate": fp64_rate,
            "gmres_cycles_per_iter": cycles / max(steps, 1)}


# drops at which the to-solution legs record iterations and seconds
MILESTONES = (1e-2, 1e-4, 1e-6, 2e-8)


def run_to_solution(w, prec, cap_s, target=1e-8, max_iters=20000, from_peak=False, **over):
    """Iterate until the rho L2 residual drops by `target` (or the time cap):
    relative to the first iteration's, or with `from_peak` to the largest seen
    (a case started from a uniform state whose residual first grows)."""
    from icsfoam_gb300 import cases, gpu

    b = gpu.binding()
    h = gpu.open_case(w.mesh, cases.make_config(b, w.settings, precision=prec, **over))
    h.set_primitive(w.p, w.U, w.T)
    t0 = time.perf_counter()
    r0 = None
    it = 0
    drop = 1.0
    best = 1.0
    hist = []
    cycles = 0
    marks = {m: None for m in MILESTONES if m > target}
    while it < max_iters:
        h.pseudo_loop()
        s = h.pseudo_iteration()
        it += 1
        cycles += s.perf.n_iterations
        r0 = max(r0 or 0.0, s.rho_l2_residual) if from_peak else (r0 or s.rho_l2_residual)
        drop = s.rho_l2_residual / r0
        best = min(best, drop)
        for m in marks:
            if marks[m] is None and drop <= m:
                marks[m] = (it, round(time.perf_counter() - t0, 3))
        if it % 100 == 0:
            hist.append((it, round(time.perf_counter() - t0, 2), drop))
        if drop <= target or time.perf_counter() - t0 > cap_s:
            break
    dt = time.perf_counter() - t0
    state = h.get_state()["W"]
    h.close()
    return {"iterations": it, "seconds": dt, "drop": drop, "min_drop": best, "reached": drop <= target,
            "cell_iters_per_s": w.mesh.n_cells * it / dt, "gmres_cycles_per_iter": cycles / max(it, 1),
            "milestones": {("%.0e" % m): v for m, v in marks.items()},
            "history": hist[::max(1, len(hist) // 12)] + hist[-1:]}, state


# Reference dictionary settings under which the pseudo-time iteration of the
# bump channel reaches a 1e-8 drop of the rho residual.  With the configured
# cellLimited<Venkatakrishnan> gradients the reference algorithm (the oracle
# as much as this GPU path) stalls: OpenFOAM's Venkatakrishnan limiter has no
# smoothing parameter and is below 1 for every finite ratio, so the face that
# sets a cell's limiter keeps switching and the residual plateaus (1e-7..1e-5
# on the 64x16x16 channel for the oracle, ~1e-3 on the 256x64x64 one).  The
# cellLimited<minmod> gradients converge on the 64x16x16 channel but stall at
# ~4e-4 on 256x64x64; the TVD vanLeer limitedScheme of the reference's
# tutorials (interpolationSchemes "reconstruct(rho) vanLeer", same for U, T)
# converges on the 64x16x16 channel and reaches ~1.3e-8 on 256x64x64 (the
# second-order leg, with its milestones down to 2e-8); first-order
# reconstruction reaches 1e-8 on both (the first-order leg).
SOLUTION_SETTINGS = {"recon_rho": 1, "recon_U": 1, "recon_T": 1}
FIRST_ORDER_SETTINGS = {"recon_rho": 0, "recon_U": 0, "recon_T": 0}
SOLUTION_SCHEME = "vanLeer (TVD limitedScheme, Gauss linear gradient)"


# The viscous box converges best with the cellLimited<minmod> gradients (a
# 3e-8 drop at 24^3 where Venkatakrishnan stalls at 1e-3 and vanLeer at 1e-1).
VISCOUS_SETTINGS = {"recon_rho": 4, "recon_U": 4, "recon_T": 4}
VISCOUS_SCHEME = "linearUpwind + cellLimited<minmod> Gauss linear 1"


def run_solution_pair(w, cap_s, settings, plateau_cap_s=0.0, from_peak=False, target=1e-8, scheme=None):
    """Mixed precision and FP64 to a 1e-8 drop under `settings`: iterations,
    seconds, sustained cell-iters/s, and the converged fields' difference;
    with plateau_cap_s > 0 also the configured reconstruction (mixed) for that
    long, to record where it stalls."""
    import numpy as np

    def rel(a, b):
        scale = np.abs(b).max(axis=0)
        scale[1:4] = scale[1:4].max()
        return float((np.abs(a - b) / scale).max())

    sm, Wm = run_to_solution(w, 1, cap_s, target=target, from_peak=from_peak, **settings)
    sd, Wd = run_to_solution(w, 0, 2.5 * cap_s, target=target, from_peak=from_peak, **settings)
    speed = {}
    for m, vm in sm["milestones"].items():
        vd = sd["milestones"].get(m)
        if vm and vd:
            speed[m] = round(vd[1] / vm[1], 3)
    out = {"scheme": scheme or SOLUTION_SCHEME, "target_drop": target, "mixed": sm, "fp64": sd,
           "mixed_speedup_to_target": (sd["seconds"] / sm["seconds"]) if sm["reached"] and sd["reached"] else None,
           "mixed_speedup_at_milestones": speed,
           "final_field_max_rel_diff": rel(Wm, Wd)}
    if plateau_cap_s > 0:
        pm, _ = run_to_solution(w, 1, plateau_cap_s, from_peak=from_peak)
        out["configured_venkatakrishnan_mixed"] = pm
    return out


def _history_worker(args):
    """The oracle's rho L2 history of one reduced workload (CPU process)."""
    name, settings, iters, every = args
    sys.path.insert(0, ROOT)
    import oracle
    from icsfoam_gb300 import cases

    w = _study_workload(name)
    h = oracle.open_case(w.mesh, cases.make_config(oracle.binding(), w.settings, **settings))
    h.set_primitive(w.p, w.U, w.T)
    hist = []
    for it in range(iters):
        h.pseudo_loop()
        s = h.pseudo_iteration()
        if it % every == 0 or it == iters - 1:
            hist.append((it, s.rho_l2_residual))
    return hist


def _study_workload(name):
    from icsfoam_gb300 import cases

    if name == "bump_64x16x16":
        return cases.bump_channel(64, 16, 16, ordering_mode="colour")
    return cases.random_box(int(name.rsplit("_", 1)[1]))


def run_convergence_study(iters=1500, every=50, runs=None):
    """rho L2 histories of the reduced bump channel (64x16x16) and viscous box
    (24^3) under the configured cellLimited<Venkatakrishnan> gradients, under
    cellLimited<minmod> and under the vanLeer limitedScheme, from the GPU
    (FP64) and from the oracle run at the same time on host cores: the two
    stall together where the algorithm stalls and converge together where it
    converges."""
    import multiprocessing as mp

    from icsfoam_gb300 import cases, gpu

    if runs is None:
        runs = [(name, label, settings) for name in ("bump_64x16x16", "random_box_24")
                for label, settings in (("venkatakrishnan", {}),
                                        ("minmod", {"recon_rho": 4, "recon_U": 4, "recon_T": 4}),
                                        ("vanleer", SOLUTION_SETTINGS))]
    ctx = mp.get_context("spawn")
    with ctx.Pool(len(runs)) as pool:
        pending = pool.map_async(_history_worker, [(n, st, iters, every) for n, _, st in runs])
        b = gpu.binding()
        gpu_hist = []
        for name, label, settings in runs:
            w = _study_workload(name)
            h = gpu.open_case(w.mesh, cases.make_config(b, w.settings, **settings))
            h.set_primitive(w.p, w.U, w.T)
            hist = []
            for it in range(iters):
                h.pseudo_loop()
                s = h.pseudo_iteration()
                if it % every == 0 or it == iters - 1:
                    hist.append((it, s.rho_l2_residual))
            h.close()
            gpu_hist.append(hist)
        ora_hist = pending.get()
    out = {}
    for (name, label, _), hg, ho in zip(runs, gpu_hist, ora_hist):
        g = [r for _, r in hg]
        o = [r for _, r in ho]
        peak_g, peak_o = max(g), max(o)
        out["%s_%s" % (name, label)] = {
            "iterations": iters,
            "gpu_min_drop_from_peak": min(g[g.index(peak_g):]) / peak_g,
            "oracle_min_drop_from_peak": min(o[o.index(peak_o):]) / peak_o,
            "gpu_last_drop": g[-1] / peak_g, "oracle_last_drop": o[-1] / peak_o,
            "history": [(it, rg, ro) for (it, rg), (_, ro) in zip(hg, ho)],
        }
    return out


def run_e2e(w, steps, warmup):
    """Through the C ABI with pinned host buffers: state H2D, one pseudo iteration, state D2H per step.

    Same warm-up and step count as the device-timed leg, so both time the
    same iterations of the same trajectory.
    """
    import numpy as np

    from icsfoam_gb300 import cases, gpu

    import torch

    b = gpu.binding()
    h = tuned(gpu.open_case(w.mesh, cases.make_config(b, w.settings, precision=1)), 1)
    h.set_primitive(w.p, w.U, w.T)
    n = w.mesh.n_cells
    # the state lives in pinned host memory between steps
    W = torch.empty((n, 5), dtype=torch.float64, pin_memory=True).numpy()
    h.get_conservative(W)
    for _ in range(warmup):
        h.set_conservative(W)
        h.pseudo_loop()
        h.pseudo_iteration()
        h.get_conservative(W)
    t0 = time.perf_counter()
    for _ in range(steps):
        h.set_conservative(W)
        h.pseudo_loop()
        s = h.pseudo_iteration()
        h.get_conservative(W)
    dt = time.perf_counter() - t0
    h.close()
    return {"value": n * steps / dt, "unit": UNIT, "h2d_bytes_per_step": int(W.nbytes),
            "d2h_bytes_per_step": int(W.nbytes + 8 * np.dtype("float64").itemsize),
            "host_buffers": "pinned"}


def run_hb_sweep(instances=(3, 5, 7, 9), per=(32, 64, 128), steps=5, warmup=2):
    """Harmonic Balance: 3/5/7/9 stacked instances of the 262,144-cell annular sector (rotational cyclic
    sides, inlet total pressure oscillating 2% at 5 kHz), mixed precision, one coupled GMRES per pseudo
    iteration."""
    from icsfoam_gb300 import cases, gpu

    b = gpu.binding()
    out = {}
    for n in instances:
        w = cases.hb_annular_sector(*per, frequency=5000.0, harmonics=(n - 1) // 2, amplitude=0.02)
        h = gpu.open_case(w.mesh, cases.make_config(b, w.settings, precision=1))
        h.set_hb(*w.hb)
        h.set_primitive(w.p, w.U, w.T)
        for _ in range(warmup):
            h.pseudo_loop()
            h.pseudo_iteration()
        h.timer_start()
        for _ in range(steps):
            h.pseudo_loop()
            h.pseudo_iteration()
        ms = h.timer_stop()
        h.close()
        out["%d_instances" % n] = {"cells": w.mesh.n_cells, "ms_per_iter": round(ms / steps, 3),
                                   "cell_iters_per_s": w.mesh.n_cells * steps / (ms / 1000.0)}
    return out


def run_batch(n_cases=64, steps=3, seed=2, precision=1, modes=("stacked", "concurrent", "sequential")):
    """64 independent shock-tube cases (Sod, AUSM+up, backward dual-time ddt, pseudo CFL 50,
    GMRES(8)+LU-SGS), N ~ U[2000, 50000] (seeded), `steps` physical time steps, each case
    pseudo-iterating until its own pseudotimeControl completes; three ways: one after another
    (the reference's way), handles iterated concurrently from host threads
    (ics_pseudo_iteration_batch), and all cases stacked in one handle (ics_set_cases: one
    launch sequence per pseudo iteration for every case).  cell-iters/s counts each case's own
    pseudo iterations (identical in the three runs, which the leg checks); a warm-up time step
    first, on fresh handles."""
    import numpy as np

    from icsfoam_gb300 import abi, cases, gpu

    b = gpu.binding()
    ws = cases.shock_tube_batch(n_cases, seed=seed)
    cells = np.array([w.mesh.n_cells for w in ws])

    def handles():
        hs = []
        for w in ws:
            h = gpu.open_case(w.mesh, cases.make_config(b, w.settings, precision=precision))
            h.set_primitive(w.p, w.U, w.T)
            hs.append(h)
        return hs

    def sequential(hs, nsteps):
        its = np.zeros(n_cases, int)
        for k, h in enumerate(hs):
            for _ in range(nsteps):
                h.begin_time_step()
                while h.pseudo_loop():
                    h.pseudo_iteration()
                    its[k] += 1
        return its

    def concurrent(hs, nsteps):
        its = np.zeros(n_cases, int)
        for _ in range(nsteps):
            for h in hs:
                h.begin_time_step()
            live = list(range(n_cases))
            while True:
                live = [k for k in live if hs[k].pseudo_loop()]
                if not live:
                    break
                abi.pseudo_iteration_batch([hs[k] for k in live])
                its[live] += 1
        return its

    wst, start = cases.stack_cases(ws)
    hst = gpu.open_case(wst.mesh, cases.make_config(b, wst.settings, precision=precision))
    hst.set_cases(start)
    hst.set_primitive(wst.p, wst.U, wst.T)

    def stacked(nsteps):
        its = np.zeros(n_cases, int)
        for _ in range(nsteps):
            hst.begin_time_step()
            while hst.pseudo_loop():
                live = ~hst.case_stats()["frozen"]
                hst.pseudo_iteration()
                its[live] += 1
        return its

    out = {"cases": n_cases, "kind": "Sod shock tubes, 1D, colour-blocked, AUSM+up first order, backward ddt",
           "cells": int(cells.sum()), "time_steps": steps, "precision": "mixed" if precision else "fp64"}
    stacked(1)  # warm-up: graph capture, first launches
    t0 = time.perf_counter()
    its_st = stacked(steps)
    t_st = time.perf_counter() - t0
    hst.close()
    work = float((cells * its_st).sum())
    out.update({"pseudo_iterations_per_case": [int(its_st.min()), int(its_st.max())],
                "stacked_cell_iters_per_s": work / t_st, "stacked_s": t_st})
    if "concurrent" not in modes:
        return out
    hs = handles()
    concurrent(hs, 1)
    t0 = time.perf_counter()
    its_co = concurrent(hs, steps)
    t_co = time.perf_counter() - t0
    for h in hs:
        h.close()
    hs = handles()
    sequential(hs, 1)
    t0 = time.perf_counter()
    its_se = sequential(hs, steps)
    t_se = time.perf_counter() - t0
    for h in hs:
        h.close()
    out.update({
        "same_iterations_all_modes": bool(np.array_equal(its_st, its_co) and np.array_equal(its_st, its_se)),
        "concurrent_cell_iters_per_s": float((cells * its_co).sum()) / t_co,
        "sequential_cell_iters_per_s": float((cells * its_se).sum()) / t_se,
        "concurrent_s": t_co, "sequential_s": t_se,
        "stacked_over_sequential": t_se / t_st, "stacked_over_concurrent": t_co / t_st})
    return out


def run_viscous_box(n=96, steps=10, warmup=3):
    """The viscous randomised box (Sutherland, isothermal wall), mixed precision
    and FP64: with the RCM numbering the config names (many LU-SGS levels:
    sync-free sweeps) and with RCM followed by colour blocking (two levels:
    the fused LU-SGS operator), each iterated from the same initial state."""
    from icsfoam_gb300 import cases, gpu

    b = gpu.binding()
    out = {}
    for order in ("rcm", "rcm+colour"):
        w = cases.random_box(n, ordering_mode=order)
        leg = {}
        for prec, name in ((1, "mixed"), (0, "fp64")):
            h = gpu.open_case(w.mesh, cases.make_config(b, w.settings, precision=prec))
            h.set_primitive(w.p, w.U, w.T)
            for _ in range(warmup):
                h.pseudo_loop()
                h.pseudo_iteration()
            h.timer_start()
            for _ in range(steps):
                h.pseudo_loop()
                h.pseudo_iteration()
            ms = h.timer_stop()
            h.close()
            leg[name] = {"ms_per_iter": round(ms / steps, 3),
                         "cell_iters_per_s": w.mesh.n_cells * steps / (ms / 1000.0)}
        leg["mixed_over_fp64"] = leg["mixed"]["cell_iters_per_s"] / leg["fp64"]["cell_iters_per_s"]
        out[order] = leg
    return {"workload": "random_box_%d" % n, "cells": w.mesh.n_cells, **out}


def run_mrf_annulus(nr=32, nt=64, nz=128, steps=10, warmup=3):
    """The 20-degree annular sector (262,144 cells) with its rotating middle third
    (MRF zone, 300 rad/s), mixed precision: one steady time step per iteration, so
    the frame velocity is re-assigned on the rotating patches each time."""
    from icsfoam_gb300 import cases, gpu
    from icsfoam_gb300 import mrf as MRF

    b = gpu.binding()
    w = cases.annular_sector(nr, nt, nz)
    h = gpu.open_case(w.mesh, cases.make_config(b, w.settings, precision=1))
    h.set_primitive(w.p, w.U, w.T)
    h.set_mrf(MRF.frame_fields(w.mesh, *w.mrf))
    first = None
    for _ in range(warmup):
        h.begin_time_step()
        s = h.pseudo_iteration()
        first = first or s.rho_l2_residual
    h.timer_start()
    for _ in range(steps):
        h.begin_time_step()
        s = h.pseudo_iteration()
    ms = h.timer_stop()
    h.close()
    return {"workload": w.name + "_mrf", "cells": w.mesh.n_cells, "ms_per_iter": round(ms / steps, 3),
            "cell_iters_per_s": w.mesh.n_cells * steps / (ms / 1000.0),
            "rho_residual_drop": s.rho_l2_residual / first}


def run_diff(nx=240, ny=128, nz=128, reps=5):
    """Residual derivatives on the swept bump: forward-mode JVP, exact Jacobian assembly by
    coloured JVPs, and the transpose product (VJP)."""
    import numpy as np

    from icsfoam_gb300 import cases, gpu

    b = gpu.binding()
    w = cases.swept_bump(nx, ny, nz)
    h = gpu.open_case(w.mesh, cases.make_config(b, w.settings))
    h.set_primitive(w.p, w.U, w.T)
    h.pseudo_iteration()
    N = w.mesh.n_cells
    v = np.random.default_rng(0).standard_normal((N, 5))
    h.jvp(v)
    h.timer_start()
    for _ in range(reps):
        h.jvp(v)
    jvp_ms = h.timer_stop() / reps
    t0 = time.perf_counter()
    nnz, ncol = h.assemble_exact_jacobian()
    asm_s = time.perf_counter() - t0
    h.vjp(v)
    h.timer_start()
    for _ in range(reps):
        h.vjp(v)
    vjp_ms = h.timer_stop() / reps
    h.close()
    out = {"workload": w.name, "cells": N, "jvp_ms": round(jvp_ms, 3), "exact_jacobian_s": round(asm_s, 3),
           "colours": ncol, "stencil_blocks": nnz, "vjp_ms": round(vjp_ms, 3),
           "note": "jvp/vjp ms include the host<->device copy of the [N,5] vectors"}
    out.update(run_adjoint(w, reps=reps))
    return out


def run_adjoint(w, iterations=3, reps=5, rel_tol=1e-8):
    """The reverse-mode VJP (gradients recomputed, no stored Jacobian) and the
    adjoint of the bump's x pressure force after some pseudo iterations:
    (V/dtau - d(R V)/dW)^T psi = dJ/dW to rel_tol, FP64 operator and FP32
    Krylov basis, transposed LU-SGS of the approximate Jacobian."""
    import numpy as np

    from icsfoam_gb300 import cases, gpu

    b = gpu.binding()
    h = gpu.open_case(w.mesh, cases.make_config(b, w.settings))
    h.set_primitive(w.p, w.U, w.T)
    for _ in range(iterations):
        h.pseudo_loop()
        h.pseudo_iteration()
    h.residual()
    h.assemble_jacobian()
    N = w.mesh.n_cells
    u = np.random.default_rng(1).standard_normal((N, 5))
    h.vjp_recompute(u)
    h.timer_start()
    for _ in range(reps):
        h.vjp_recompute(u)
    rev_ms = h.timer_stop() / reps
    bump = [p.name for p in w.mesh.patches].index("bump")
    force, g = h.pressure_force(bump, (1.0, 0.0, 0.0))
    t0 = time.perf_counter()
    psi, r = h.adjoint_solve(g, n_directions=40, max_cycles=100, rel_tol=rel_tol, precision=1, pseudo_time=1)
    adj_s = time.perf_counter() - t0
    h.close()
    return {"vjp_recompute_ms": round(rev_ms, 3), "pressure_force_x": force,
            "adjoint": {"operator": "V/dtau - d(R V)/dW (reverse mode), FP32 Krylov basis, transposed LU-SGS",
                        "iterations": r.iterations, "cycles": r.cycles, "rel_residual": r.rel_residual,
                        "converged": bool(r.converged), "seconds": round(adj_s, 3),
                        "ms_per_iteration": round(1000 * adj_s / max(r.iterations, 1), 3)}}


def _oracle_worker(args):
    """One oracle process on its own copy of the mesh: warm-up, barrier, timed iterations."""
    dims, steps, warmup, seconds, barrier = args
    sys.path.insert(0, ROOT)
    import oracle
    from icsfoam_gb300 import cases

    w = cases.bump_channel(*dims, ordering_mode="colour")
    h = oracle.open_case(w.mesh, cases.make_config(oracle.binding(), w.settings))
    h.set_primitive(w.p, w.U, w.T)
    for _ in range(warmup):
        h.pseudo_loop()
        h.pseudo_iteration()
    barrier.wait()
    t0 = time.perf_counter()
    it = 0
    while True:
        h.pseudo_loop()
        h.pseudo_iteration()
        it += 1
        if (steps and it >= steps) or (seconds and time.perf_counter() - t0 >= seconds):
            break
    return w.mesh.n_cells * it, time.perf_counter() - t0, it


def oracle_throughput(dims, steps=0, warmup=1, seconds=0.0, procs=None):
    """The oracle (the reference algorithm, FP64, single-threaded as each MPI
    rank of the reference is) on every host core, each process iterating its
    own copy of the whole mesh, started together: cell-iters/s = all cells x
    iterations / the slowest process's time.  The reference's own parallel
    run would split the mesh into as many subdomains with halo exchanges and
    allreduces (and block-Jacobi LU-SGS across them), so this aggregate is an
    upper bound of what the host cores deliver on the workload."""
    import multiprocessing as mp

    procs = procs or os.cpu_count() or 1
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    barrier = mgr.Barrier(procs)
    with ctx.Pool(procs) as pool:
        res = pool.map(_oracle_worker, [(dims, steps, warmup, seconds, barrier) for _ in range(procs)])
    work = sum(r[0] for r in res)
    dt = max(r[1] for r in res)
    its = min(r[2] for r in res)
    return work / dt, dt, procs, its


def _reference_sample(dims, procs, its, warm):
    return ("bump channel %dx%dx%d (the timed workload itself), one copy per host core (%d processes, "
            "single-threaded each) of >= %d pseudo iterations after %d warm-up; HLLC MUSCL/Venkatakrishnan, "
            "GMRES(8)+LU-SGS, FP64 oracle; aggregate of independent full-mesh runs = an upper bound of a "
            "%d-subdomain decomposed run" % (dims + (procs, its, warm, procs)))


def cpu_sample(dims, seconds, warm=1):
    """The oracle on all host cores for about ``seconds`` (bounded sample)."""
    v, dt, procs, its = oracle_throughput(dims, seconds=seconds, warmup=warm)
    return {"value": v, "unit": UNIT, "cores": procs, "kind": "port",
            "sample": _reference_sample(dims, procs, its, warm)}


def reference_arm(args, dist):
    if dist.rank != 0:
        return
    dims = (args.nx, args.ny, args.nz)
    v, dt, procs, its = oracle_throughput(dims, steps=args.steps, warmup=args.warmup)
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * dt / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (generated bump-channel mesh, uniform M=0.675 initial state)",
            "config": {"workload": "bump_channel_%dx%dx%d" % dims, "cells": args.nx * args.ny * args.nz,
                       "processes": procs, "flux": "HLLC",
                       "reconstruction": "MUSCL + cellLimited<Venkatakrishnan>", "solver": "GMRES(8)+LU-SGS",
                       "ordering": "colour-blocked"},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": procs, "kind": "port",
                             "sample": _reference_sample(dims, procs, its, args.warmup)},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    dist = Dist(args.gpus)
    if args.impl == "reference":
        reference_arm(args, dist)
        dist.close()
        return
    if dist.world > 1:
        os.environ["CUDA_VISIBLE_DEVICES"] = str(dist.local)
    from icsfoam_gb300 import cases

    if args.batch:
        # the independent-case batch alone (stacked only with --batch-stacked-only 1)
        modes = ("stacked",) if args.batch_stacked_only else ("stacked", "concurrent", "sequential")
        print(json.dumps(run_batch(n_cases=args.batch, modes=modes)), flush=True)
        dist.close()
        return
    if args.adjoint:
        w = cases.swept_bump(240, 128, 128)
        print(json.dumps({"workload": w.name, "cells": w.mesh.n_cells, **run_adjoint(w)}), flush=True)
        dist.close()
        return
    if args.convergence_study:
        runs = None
        if args.study_box_first:
            # the viscous box with first-order reconstruction, GPU and oracle in lockstep
            runs = [("random_box_%d" % args.study_box_first, "first_order", FIRST_ORDER_SETTINGS)]
        print(json.dumps({"convergence_study": run_convergence_study(args.convergence_study, runs=runs)}), flush=True)
        dist.close()
        return
    if args.viscous_solution:
        # the randomised viscous box at its configured size and numbering (RCM)
        w = cases.random_box(200)
        res = run_solution_pair(w, args.solution_cap_s, VISCOUS_SETTINGS, from_peak=True,
                                target=args.viscous_target, scheme=VISCOUS_SCHEME)
        print(json.dumps({"workload": w.name, "cells": w.mesh.n_cells, "ordering": "rcm", **res}), flush=True)
        dist.close()
        return
    t0 = time.time()
    w = cases.bump_channel(args.nx, args.ny, args.nz, ordering_mode="colour")
    mesh_s = time.time() - t0
    N, F, B = w.mesh.n_cells, w.mesh.n_faces, w.mesh.n_bfaces
    mixed = run_timed(w, 1, args.steps, args.warmup, dist, args.profile, args.autotune)
    fp64 = run_timed(w, 0, args.steps, args.warmup, dist, args.profile, args.autotune)
    value = N * args.steps * dist.world / (mixed["ms"] / 1000.0)
    value64 = N * args.steps * dist.world / (fp64["ms"] / 1000.0)
    extra = {}
    # the long single-GPU legs run only in a 1-GPU run: a scaling run holds all
    # N GPUs while rank 0 would run them
    if dist.rank == 0 and args.to_solution and dist.world == 1:
        # first-order reconstruction reaches 1e-8 in both precisions; the
        # second-order vanLeer one stalls at ~1.3e-8 on this mesh (milestones
        # to 2e-8); the configured Venkatakrishnan limiter's plateau recorded
        first = run_solution_pair(w, args.solution_cap_s, FIRST_ORDER_SETTINGS, scheme="upwind (first order)")
        second = run_solution_pair(w, args.solution_cap_s, SOLUTION_SETTINGS, plateau_cap_s=args.plateau_cap_s)
        extra["to_solution"] = {"first_order": first, "second_order": second}
    e2e = run_e2e(w, args.steps, args.warmup) if dist.rank == 0 else None
    if dist.rank == 0 and args.extras and dist.world == 1:
        extra["harmonic_balance"] = run_hb_sweep()
        extra["batch_independent_cases"] = run_batch()
        extra["derivatives"] = run_diff()
        extra["viscous_box"] = run_viscous_box()
        extra["mrf_annulus"] = run_mrf_annulus()
    # roofline of the dominant kernel class of the mixed leg
    from icsfoam_gb300 import ordering  # noqa: F401

    nslots = None
    roof = None
    fp64_roof = None
    kern_table = {}
    if mixed["kernels"]:
        peak, peak_kind = load_peaks()
        traffic = load_traffic()
        fp64_peak = mixed["fp64_rate"]
        nlev = 2
        tot = sum(v[0] for v in mixed["kernels"].values())
        dom = max(mixed["kernels"].items(), key=lambda kv: kv[1][0])
        for k, (ms, n) in mixed["kernels"].items():
            if n:
                kern_table[k] = {"ms_total": round(ms, 3), "launches": n, "share": round(ms / tot, 4),
                                 "ms_per_launch": round(ms / n, 5), "bound": kernel_bound(k, True)}
                byts = kernel_bytes(k, N, F, B, nslots, True, nlev)
                if byts:
                    kern_table[k]["GBps"] = round(byts / (ms / n / 1000.0) / 1e9, 1)
                if k in FP64_FLOPS_PER_UNIT:
                    units = F if k == "face" else N
                    kern_table[k]["fp64_GFLOPs"] = round(FP64_FLOPS_PER_UNIT[k] * units / (ms / n / 1000.0) / 1e9, 1)
        # the HBM roofline of the dominant HBM-bound kernel class; the
        # FP64-bound classes get theirs against the measured FP64 FMA rate
        hbm = [(k, v) for k, v in mixed["kernels"].items() if v[1] and kernel_bound(k, True) == "hbm"
               and kernel_bytes(k, N, F, B, nslots, True, nlev)]
        name, (ms, n) = max(hbm, key=lambda kv: kv[1][0])
        byts = kernel_bytes(name, N, F, B, nslots, True, nlev)
        ach = byts / (ms / n / 1000.0) / 1e9
        tr = traffic.get((name, "mixed"))
        roof = {"kernel": name, "bound": "hbm", "achieved": round(ach, 1), "peak": peak, "unit": "GB/s",
                "frac": round(ach / peak, 4), "peak_source": peak_kind,
                "algorithmic_bytes_per_launch": int(byts),
                "traffic": (tr[1] * N / tr[0]) if tr else None,
                "share_of_step": round(ms / tot, 4),
                "dominant_kernel_overall": {"kernel": dom[0], "bound": kernel_bound(dom[0], True),
                                            "share_of_step": round(dom[1][0] / tot, 4)}}
        fp64_roof = {}
        for k in FP64_FLOPS_PER_UNIT:
            if k in mixed["kernels"] and mixed["kernels"][k][1]:
                ms_k, n_k = mixed["kernels"][k]
                units = F if k == "face" else N
                ach64 = FP64_FLOPS_PER_UNIT[k] * units / (ms_k / n_k / 1000.0) / 1e9
                trk = traffic.get((k, "fp64"))
                fp64_roof[k] = {"bound": "fp64", "achieved": round(ach64, 1), "peak": round(fp64_peak, 1),
                                "unit": "GFLOP/s", "frac": round(ach64 / fp64_peak, 4) if fp64_peak else None,
                                "peak_source": "measured FP64 FMA microkernel (ics_measure_fp64_rate)",
                                "flops_per_launch": int(FP64_FLOPS_PER_UNIT[k] * units),
                                "hbm_GBps": kern_table[k].get("GBps"),
                                "traffic": (trk[1] * N / trk[0]) if trk else None,
                                "share_of_step": round(ms_k / tot, 4)}
    fp64_table = {}
    if fp64["kernels"]:
        for k, (ms, n) in fp64["kernels"].items():
            if n:
                fp64_table[k] = {"ms_total": round(ms, 3), "launches": n}
                byts = kernel_bytes(k, N, F, B, nslots, False, 2)
                if byts:
                    fp64_table[k]["GBps"] = round(byts / (ms / n / 1000.0) / 1e9, 1)
    # the CPU baseline: rank 0 of a 1-GPU run only
    cpu = cpu_sample((args.nx, args.ny, args.nz), args.cpu_seconds) if dist.rank == 0 and dist.world == 1 else None
    if dist.rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": dist.world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": mixed["ms"] / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64 residual/update + f32 Jacobian/Krylov",
            "data": "synthetic (generated bump-channel mesh, uniform M=0.675 initial state)",
            "config": {"workload": "bump_channel_%dx%dx%d" % (args.nx, args.ny, args.nz), "cells": N,
                       "internal_faces": F, "boundary_faces": B, "flux": "HLLC",
                       "reconstruction": "MUSCL + cellLimited<Venkatakrishnan>", "solver": "GMRES(8)+LU-SGS",
                       "ordering": "colour-blocked", "parallelism": "replicas" if dist.world > 1 else "1 GPU",
                       "l2": "working set >> 129 MB L2; no flush needed",
                       "tuning": {("mixed" if k else "fp64"): v for k, v in TUNING.items()}},
            "fp64": {"value": value64, "unit": UNIT, "ms_per_step": fp64["ms"] / args.steps,
                     "gmres_cycles_per_iter": fp64["gmres_cycles_per_iter"], "kernels": fp64_table},
            "gmres_cycles_per_iter": mixed["gmres_cycles_per_iter"],
            "mixed_over_fp64": value / value64,
            "kernels": kern_table, "roofline": roof, "fp64_roofline": fp64_roof, "cpu_baseline": cpu, "e2e": e2e,
            "gpu_launches": mixed["launches"], "clocks": mixed["clocks"], "mesh_build_s": round(mesh_s, 1),
        }
        line.update(extra)
        print(json.dumps(line), flush=True)
    dist.close()


if __name__ == "__main__":
    main()
