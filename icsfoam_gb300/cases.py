"""Synthetic workloads: meshes, patches, initial fields and solver settings.

The reference is quoted on cases that are not shipped with it, so every mesh
here is generated from fixed seeds:

* ``shock_tube``   - 1D Sod problem, hex cells one thick, empty sides.
* ``bump_channel`` - 3D inviscid channel with a circular-arc bump on the
                     lower wall, total-pressure inlet and static-pressure
                     outlet, slip walls (the transonic circularArcBump layout).
* ``random_box``   - hex box with randomly displaced interior vertices, cells
                     randomly permuted then reverse-Cuthill-McKee renumbered.
* ``swept_bump``   - transonic channel over a 30-degree swept 8% bump at
                     3 degrees incidence (the differentiation workload).
* ``hb_bump_channel`` - Harmonic Balance version of the bump channel: a
                     time-periodic outlet static pressure, 2H+1 stacked
                     instances and the spectral operator D.
* ``annular_sector`` - axial flow through a 20-degree annular sector with a
                     rotational cyclic side pair and a rotating (MRF) cell
                     zone in its middle third; ``hb_annular_sector`` its
                     Harmonic Balance version (oscillating inlet total
                     pressure).

Sizes are parameters; the headline sizes are 1000 cells, 256x64x64 and 200^3.
"""

from __future__ import annotations

import dataclasses
from typing import Dict, Optional

import numpy as np

from . import mesh as M
from . import ordering


@dataclasses.dataclass
class Workload:
    name: str
    mesh: M.Mesh
    p: np.ndarray
    U: np.ndarray
    T: np.ndarray
    settings: Dict  # ics_config field overrides
    hb: Optional[tuple] = None  # Harmonic Balance (n_instances, D) or None
    mrf: Optional[tuple] = None  # moving frames: (rotating zones, translating zones) or None


GAMMA = 1.4
R_GAS = 287.0
CP = GAMMA * R_GAS / (GAMMA - 1.0)   # 1004.5


def thermo_settings():
    return {"R": R_GAS, "Cp": CP}


def shock_tube(n: int = 1000, x0: float = -5.0, x1: float = 5.0, ordering_mode: str = "natural") -> Workload:
    """Sod shock tube: left p=1e5 T=348.4, right p=1e4 T=278.7, u=0."""
    xs = np.linspace(x0, x1, n + 1)
    g = np.zeros((n + 1, 2, 2, 3))
    g[..., 0] = xs[:, None, None]
    g[:, 1, :, 1] = 1.0 * (x1 - x0) / n
    g[:, :, 1, 2] = 1.0 * (x1 - x0) / n
    ends = M.Patch("sides", M.PATCH_ZERO_GRADIENT)
    empty = M.Patch("empty", M.PATCH_EMPTY)
    sides = {"xmin": ends, "xmax": ends, "ymin": empty, "ymax": empty, "zmin": empty, "zmax": empty}
    mesh = M.hex_mesh(g, sides)
    mesh = ordering.apply(mesh, ordering_mode)
    x = mesh.C[:, 0]
    left = x < 0.0
    p = np.where(left, 1.0e5, 1.0e4)
    T = np.where(left, 348.4, 278.7)
    U = np.zeros((mesh.n_cells, 3))
    settings = dict(thermo_settings(), flux_scheme=0, ddt_scheme=2, delta_t=1e-5,
                    pseudo_co_num=50.0, pseudo_co_num_max=50.0, n_pseudo_corr=10,
                    pseudo_tol=1e-5, pseudo_tol_rel=1e-5,
                    n_directions=8, max_iter=20, tolerance=1e-12, rel_tol=1e-4)
    return Workload("shock_tube_%d" % n, mesh, p, U, T, settings)


def bump_points(nx: int, ny: int, nz: int, length=3.0, height=1.0, width=0.5, thickness=0.1) -> np.ndarray:
    """Grid points of a channel x in [-1, 2] with a circular-arc bump on x in [0, 1]."""
    xs = np.linspace(-1.0, -1.0 + length, nx + 1)
    Rb = (0.25 + thickness ** 2) / (2.0 * thickness)
    yb = np.where((xs > 0.0) & (xs < 1.0), np.sqrt(np.maximum(Rb ** 2 - (xs - 0.5) ** 2, 0.0)) - (Rb - thickness), 0.0)
    eta = np.linspace(0.0, 1.0, ny + 1)
    zs = np.linspace(0.0, width, nz + 1)
    g = np.zeros((nx + 1, ny + 1, nz + 1, 3))
    g[..., 0] = xs[:, None, None]
    g[..., 1] = (yb[:, None] + eta[None, :] * (height - yb[:, None]))[:, :, None]
    g[..., 2] = zs[None, None, :]
    return g


def bump_channel(nx: int = 256, ny: int = 64, nz: int = 64, mach: float = 0.675, p0: float = 1.0e5,
                 T0: float = 300.0, ordering_mode: str = "colour", second_order: bool = True,
                 flux: str = "HLLC") -> Workload:
    """Inviscid transonic channel over a 10% circular-arc bump (M=0.675)."""
    g = bump_points(nx, ny, nz)
    fac = 1.0 + 0.5 * (GAMMA - 1.0) * mach ** 2
    p_static = p0 / fac ** (GAMMA / (GAMMA - 1.0))
    T_static = T0 / fac
    inlet = M.Patch("inlet", M.PATCH_TOTAL_INLET, p0=p0, T0=T0)
    outlet = M.Patch("outlet", M.PATCH_PRESSURE_OUTLET, p=p_static)
    wall = M.Patch("walls", M.PATCH_SLIP, is_wall=True)
    sides = {"xmin": inlet, "xmax": outlet, "ymin": wall, "ymax": wall, "zmin": wall, "zmax": wall}
    mesh = M.hex_mesh(g, sides)
    mesh = ordering.apply(mesh, ordering_mode)
    N = mesh.n_cells
    c = np.sqrt(GAMMA * R_GAS * T_static)
    p = np.full(N, p_static)
    T = np.full(N, T_static)
    U = np.zeros((N, 3))
    U[:, 0] = mach * c
    rec = 3 if second_order else 0
    settings = dict(thermo_settings(), flux_scheme={"AUSMPlusUp": 0, "HLLC": 1, "ROE": 2}[flux],
                    recon_rho=rec, recon_U=rec, recon_T=rec,
                    ddt_scheme=0, pseudo_co_num=1.0, pseudo_co_num_max=200.0,
                    n_directions=8, max_iter=5, tolerance=1e-12, rel_tol=1e-2,
                    pseudo_tol=1e-30, pseudo_tol_rel=1e-30)
    return Workload("bump_%dx%dx%d" % (nx, ny, nz), mesh, p, U, T, settings)


def random_box(n: int = 200, seed_vertices: int = 0, seed_perm: int = 1, mach: float = 2.0,
               p: float = 1.0e4, T: float = 220.0, T_wall: float = 300.0, length: float = 1.0,
               ordering_mode: str = "rcm", jitter: float = 0.2, reynolds_per_m: float = 1.0e5) -> Workload:
    """Randomised hex box: interior vertices displaced by U(+-jitter h), cells permuted then RCM.

    Viscous supersonic flow over an isothermal wall (bottom): Sutherland
    viscosity scaled so that rho U / mu equals ``reynolds_per_m`` in the
    freestream, Pr = 0.72.
    """
    h = length / n
    xs = np.linspace(0.0, length, n + 1)
    g = np.stack(np.meshgrid(xs, xs, xs, indexing="ij"), axis=-1)
    rng = np.random.default_rng(seed_vertices)
    disp = rng.uniform(-jitter * h, jitter * h, size=g.shape)
    interior = np.zeros(g.shape[:3], bool)
    interior[1:-1, 1:-1, 1:-1] = True
    g = g + np.where(interior[..., None], disp, 0.0)
    c = np.sqrt(GAMMA * R_GAS * T)
    uinf = mach * c
    inlet = M.Patch("inlet", M.PATCH_FIXED, p=p, T=T, U=(uinf, 0.0, 0.0))
    outlet = M.Patch("outlet", M.PATCH_ZERO_GRADIENT)
    wall = M.Patch("wall", M.PATCH_ISOTHERMAL_WALL, is_wall=True, T=T_wall)
    top = M.Patch("top", M.PATCH_ZERO_GRADIENT)
    sym = M.Patch("sides", M.PATCH_SLIP)
    sides = {"xmin": inlet, "xmax": outlet, "ymin": wall, "ymax": top, "zmin": sym, "zmax": sym}
    mesh = M.hex_mesh(g, sides)
    perm = np.random.default_rng(seed_perm).permutation(mesh.n_cells)
    mesh = M.renumber(mesh, perm)
    mesh = ordering.apply(mesh, ordering_mode)
    N = mesh.n_cells
    Uc = np.zeros((N, 3))
    Uc[:, 0] = uinf
    # Sutherland constant As chosen so that rho u / mu(T) = Re per metre
    rho = p / (R_GAS * T)
    Ts = 110.4
    mu_inf = rho * uinf / reynolds_per_m
    As = mu_inf * (1.0 + Ts / T) / np.sqrt(T)
    settings = dict(thermo_settings(), flux_scheme=0, recon_rho=3, recon_U=3, recon_T=3,
                    ddt_scheme=0, pseudo_co_num=1.0, pseudo_co_num_max=50.0,
                    n_directions=8, max_iter=5, rel_tol=1e-2, tolerance=1e-12,
                    pseudo_tol=1e-30, pseudo_tol_rel=1e-30,
                    viscous=1, sutherland=1, As=float(As), Ts=Ts, Pr=0.72)
    return Workload("random_box_%d" % n, mesh, np.full(N, p), Uc, np.full(N, T), settings)


def swept_bump(nx: int = 240, ny: int = 128, nz: int = 128, thickness: float = 0.08, sweep_deg: float = 30.0,
               mach: float = 0.84, alpha_deg: float = 3.0, p0: float = 1.0e5, T0: float = 300.0,
               ordering_mode: str = "colour", flux: str = "HLLC") -> Workload:
    """Transonic channel over a swept circular-arc bump (the differentiation case).

    The 8% arc spans x in [s, s+1] with s = z tan(sweep), so its crest line is
    swept by ``sweep_deg`` across the span; the initial flow is uniform at
    M = 0.84 inclined by ``alpha_deg`` in the x-y plane.
    """
    length, height, width = 3.0, 1.0, 1.0
    xs = np.linspace(-1.0, -1.0 + length, nx + 1)
    eta = np.linspace(0.0, 1.0, ny + 1)
    zs = np.linspace(0.0, width, nz + 1)
    Rb = (0.25 + thickness ** 2) / (2.0 * thickness)
    shift = zs * np.tan(np.radians(sweep_deg))
    xl = xs[:, None] - shift[None, :]
    yb = np.where((xl > 0.0) & (xl < 1.0), np.sqrt(np.maximum(Rb ** 2 - (xl - 0.5) ** 2, 0.0)) - (Rb - thickness), 0.0)
    g = np.zeros((nx + 1, ny + 1, nz + 1, 3))
    g[..., 0] = xs[:, None, None]
    g[..., 1] = yb[:, None, :] + eta[None, :, None] * (height - yb[:, None, :])
    g[..., 2] = zs[None, None, :]
    fac = 1.0 + 0.5 * (GAMMA - 1.0) * mach ** 2
    p_static = p0 / fac ** (GAMMA / (GAMMA - 1.0))
    T_static = T0 / fac
    inlet = M.Patch("inlet", M.PATCH_TOTAL_INLET, p0=p0, T0=T0)
    outlet = M.Patch("outlet", M.PATCH_PRESSURE_OUTLET, p=p_static)
    wall = M.Patch("walls", M.PATCH_SLIP, is_wall=True)
    bump = M.Patch("bump", M.PATCH_SLIP, is_wall=True)  # the lower wall carrying the swept bump
    sides = {"xmin": inlet, "xmax": outlet, "ymin": bump, "ymax": wall, "zmin": wall, "zmax": wall}
    mesh = M.hex_mesh(g, sides)
    mesh = ordering.apply(mesh, ordering_mode)
    N = mesh.n_cells
    c = np.sqrt(GAMMA * R_GAS * T_static)
    a = np.radians(alpha_deg)
    U = np.zeros((N, 3))
    U[:, 0] = mach * c * np.cos(a)
    U[:, 1] = mach * c * np.sin(a)
    settings = dict(thermo_settings(), flux_scheme={"AUSMPlusUp": 0, "HLLC": 1, "ROE": 2}[flux],
                    recon_rho=3, recon_U=3, recon_T=3, ddt_scheme=0, pseudo_co_num=1.0,
                    pseudo_co_num_max=200.0, n_directions=8, max_iter=5, tolerance=1e-12, rel_tol=1e-2,
                    pseudo_tol=1e-30, pseudo_tol_rel=1e-30)
    return Workload("swept_bump_%dx%dx%d" % (nx, ny, nz), mesh, np.full(N, p_static), U, np.full(N, T_static),
                    settings)


def hb_bump_channel(nx: int = 64, ny: int = 16, nz: int = 4, frequency: float = 50.0, harmonics: int = 1,
                    amplitude: float = 0.05, selected_period: Optional[float] = None, **kw) -> Workload:
    """Bump channel under an oscillating back pressure p_out (1 + a sin(w t)).

    Instance J is the flow at instant t_J: its outlet patch carries
    p_out(t_J); the instants are equispaced over ``selected_period`` or, when
    None, over the period of smallest condition number (HBZoneList::setInstants).
    """
    from . import hb as HB
    w = bump_channel(nx, ny, nz, **kw)
    omegas = HB.omega_list([2.0 * np.pi * frequency], [harmonics])
    n = 2 * harmonics + 1
    t = HB.select_instants(omegas, n, selected_period)
    D = HB.hb_operator(omegas, t)
    p_out = next(p.p for p in w.mesh.patches if p.kind == M.PATCH_PRESSURE_OUTLET)

    def patch_for(q, J):
        if q.kind == M.PATCH_PRESSURE_OUTLET:
            q.p = p_out * (1.0 + amplitude * np.sin(omegas[1] * t[J]))
        return q

    st = HB.stack_instances(w.mesh, n, patch_for)
    rep = lambda a: np.concatenate([a] * n)
    return Workload("hb%d_%s" % (n, w.name), st, rep(w.p), rep(w.U), rep(w.T), dict(w.settings), hb=(n, D))


def annular_sector(nr: int = 32, nt: int = 64, nz: int = 128, r0: float = 0.5, r1: float = 0.6,
                   sector_deg: float = 20.0, length: float = 0.2, mach: float = 0.4, omega: float = 300.0,
                   p0: float = 1.0e5, T0: float = 300.0, ordering_mode: str = "colour", flux: str = "HLLC",
                   second_order: bool = True, sides: str = "cyclic", theta0_deg: Optional[float] = None) -> Workload:
    """Axial flow through an annular sector r in [r0, r1], theta in
    [theta0, theta0 + sector] (theta0 = -sector/2 by default), z in [0,
    length]: total-pressure inlet (z = 0), static-pressure outlet, slip hub
    and shroud walls; the sector's side planes are a rotational cyclic pair
    (``sides="cyclic"``: "sideA" at theta0 couples to "sideB" rotated by
    -sector about z) or slip planes (``sides="slip"``, patch "sides").  The
    cells with z in [length/3, 2 length/3] form a zone rotating at ``omega``
    rad/s about the z axis (an MRFProperties zone; the cyclic sides are its
    coupled patches).  Cell index order: i radial, j circumferential, k axial."""
    from . import mrf as MRF
    rs = np.linspace(r0, r1, nr + 1)
    t0 = -0.5 * sector_deg if theta0_deg is None else theta0_deg
    th = np.radians(np.linspace(t0, t0 + sector_deg, nt + 1))
    zs = np.linspace(0.0, length, nz + 1)
    g = np.zeros((nr + 1, nt + 1, nz + 1, 3))
    g[..., 0] = rs[:, None, None] * np.cos(th)[None, :, None]
    g[..., 1] = rs[:, None, None] * np.sin(th)[None, :, None]
    g[..., 2] = zs[None, None, :]
    fac = 1.0 + 0.5 * (GAMMA - 1.0) * mach ** 2
    p_static = p0 / fac ** (GAMMA / (GAMMA - 1.0))
    T_static = T0 / fac
    inlet = M.Patch("inlet", M.PATCH_TOTAL_INLET, p0=p0, T0=T0)
    outlet = M.Patch("outlet", M.PATCH_PRESSURE_OUTLET, p=p_static)
    hub = M.Patch("hub", M.PATCH_SLIP, is_wall=True)
    shroud = M.Patch("shroud", M.PATCH_SLIP, is_wall=True)
    if sides == "cyclic":
        sa, sb = M.cyclic_pair("sideA", "sideB", (0.0, 0.0, 1.0), -sector_deg)
        coupled = ("sideA", "sideB")
    else:
        sa = sb = M.Patch("sides", M.PATCH_SLIP)
        coupled = ()
    side_map = {"xmin": hub, "xmax": shroud, "ymin": sa, "ymax": sb, "zmin": inlet, "zmax": outlet}
    mesh = M.hex_mesh(g, side_map)
    mesh = ordering.apply(mesh, ordering_mode)
    N = mesh.n_cells
    c = np.sqrt(GAMMA * R_GAS * T_static)
    U = np.zeros((N, 3))
    U[:, 2] = mach * c
    zc = mesh.C[:, 2]
    rotor = (zc > length / 3.0) & (zc < 2.0 * length / 3.0)
    zone = MRF.RotatingZone(cells=rotor, origin=(0.0, 0.0, 0.0), axis=(0.0, 0.0, 1.0), omega=omega,
                            coupled_patches=coupled)
    rec = 3 if second_order else 0
    settings = dict(thermo_settings(), flux_scheme={"AUSMPlusUp": 0, "HLLC": 1, "ROE": 2}[flux],
                    recon_rho=rec, recon_U=rec, recon_T=rec, ddt_scheme=0, pseudo_co_num=1.0,
                    pseudo_co_num_max=200.0, n_directions=8, max_iter=5, tolerance=1e-12, rel_tol=1e-2,
                    pseudo_tol=1e-30, pseudo_tol_rel=1e-30)
    return Workload("annulus_%dx%dx%d%s" % (nr, nt, nz, "" if sides == "cyclic" else "_slip"), mesh, np.full(N, p_static), U, np.full(N, T_static),
                    settings, mrf=([zone], []))


def hb_annular_sector(nr: int = 32, nt: int = 64, nz: int = 128, frequency: float = 5000.0, harmonics: int = 1,
                      amplitude: float = 0.02, selected_period: Optional[float] = None, **kw) -> Workload:
    """Harmonic Balance on the rotational-cyclic annular sector: the inlet
    total pressure oscillates, p0 (1 + a sin(2 pi f t)); 2H+1 stacked
    instances of ``annular_sector`` (the rotating zone is not applied)."""
    from . import hb as HB
    w = annular_sector(nr, nt, nz, **kw)
    omegas = HB.omega_list([2.0 * np.pi * frequency], [harmonics])
    n = 2 * harmonics + 1
    t = HB.select_instants(omegas, n, selected_period)
    D = HB.hb_operator(omegas, t)

    def patch_for(q, J):
        if q.kind == M.PATCH_TOTAL_INLET:
            q.p0 = q.p0 * (1.0 + amplitude * np.sin(omegas[1] * t[J]))
        return q

    st = HB.stack_instances(w.mesh, n, patch_for)
    rep = lambda a: np.concatenate([a] * n)
    return Workload("hb%d_%s" % (n, w.name), st, rep(w.p), rep(w.U), rep(w.T), dict(w.settings), hb=(n, D))


def make_config(binding, settings: Dict, **overrides):
    cfg = binding.default_config()
    for k, v in dict(settings, **overrides).items():
        setattr(cfg, k, v)
    return cfg


def stack_cases(workloads) -> "tuple[Workload, np.ndarray]":
    """Independent cases as one stacked workload (mesh.stack) with the case
    offsets for CaseHandle.set_cases.  The cases share one solver
    configuration: the first workload's settings."""
    mesh, start = M.stack([w.mesh for w in workloads])
    w0 = workloads[0]
    cat = lambda f: np.concatenate([f(w) for w in workloads])
    w = Workload("stack_%d" % len(workloads), mesh, cat(lambda w: w.p), cat(lambda w: w.U), cat(lambda w: w.T),
                 dict(w0.settings))
    return w, start


def shock_tube_batch(n_cases: int = 64, seed: int = 2, low: int = 2000, high: int = 50000, ordering_mode="colour"):
    """The many-small-cases batch: Sod shock tubes with cell counts drawn
    uniformly from [low, high] (seeded), each over x in [-5, 5]."""
    rng = np.random.default_rng(seed)
    sizes = rng.integers(low, high + 1, n_cases)
    return [shock_tube(int(n), ordering_mode=ordering_mode) for n in sizes]
