"""Synthetic problem setups with the shapes of the five benchmark configurations.

Every setup is deterministic (config 4 draws from our own splitmix64 stream
with seed 0x5EED2026).  Initial states follow the reference initialisers'
semantics (init/InitTwoFluidShockTube.cpp, init/InitShockBubble.cpp,
init/InitDropletAdvection.cpp, init/InitTriplePoint.cpp): per-region
primitive states (alpha_0, alpha_rho_k, p, velocity) converted to the
conservative vector with the stiffened-gas mixture EOS.

Variable ids (models/FiveEq.h:35-50): 2D ID=0 IE=1 IU=2 IV=3 IA0=4 IAD0=5
IA1=6 IAD1=7; 3D adds IW=4 and shifts the material ids by one.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from .mesh import BC_PERIODIC, BC_WALL, BC_ZERO_GRADIENT, BlockMesh, BlockTable, cell_centers, concat_tables

INTEGRATOR = {"HANCOCK": 0, "RK1": 1, "RK2_SSP": 2}
SOURCE_TERM = {"ALLAIRE_KOKH": 0, "MILLER_PUCKETT": 1}
INDICATOR = {"SIMPLE_GRADIENT": 0, "LOHNER_UNSPLIT": 1, "LOHNER_SPLIT": 2}


def ids(dim: int) -> dict:
    hc = 4 if dim == 2 else 5
    d = {"ID": 0, "IE": 1, "IP": 1, "IU": 2, "IV": 3, "IA0": hc, "IAD0": hc + 1, "IA1": hc + 2, "IAD1": hc + 3, "NV": hc + 4}
    d["IW"] = 4 if dim == 3 else 3
    return d


@dataclass
class HydroParams:
    """Scheme parameters (HydroSettings, THINCParams, time integrator, EOS, BCs)."""

    dim: int = 2
    bsize: int = 16
    gamma: tuple = (1.4, 1.4)
    pinf: tuple = (0.0, 0.0)
    smallr: float = 1e-10  # models/HydroSettings.cpp:18-29 defaults
    smallc: float = 1e-10
    slope_type: float = 1.0
    cfl: float = 0.5
    integrator: int = 0  # HANCOCK
    thinc: int = 0
    thinc_beta: float = 1.6
    thinc_eps: float = 1e-3
    source_term: int = 0  # ALLAIRE_KOKH
    prolongation: int = 0  # SIMPLE_COPY
    bc: tuple = (BC_PERIODIC,) * 6
    level_dx: np.ndarray = field(default_factory=lambda: np.zeros(32))
    # material laws: EOS_* per material and the law parameters (G5Params.mg)
    eos: tuple = (0, 0)
    mg: tuple = ((0.0,) * 8, (0.0,) * 8)


# material laws (G5Params.eos / .mg); the device and the oracle restate them
EOS = {"STIFFENED": 0, "JWL": 1, "SHOCKWAVE": 2, "SHOCKWAVE2": 3}


def mg_law(params: HydroParams, k: int, rho):
    """G(rho) and f(rho) of material k's law written p = G rho e + f (numpy;
    initial states only)."""
    rho = np.asarray(rho, dtype=np.float64)
    kind, c = params.eos[k], params.mg[k]
    if kind == EOS["JWL"]:
        rho0, w, A1, A2, R1, R2, e0 = c[:7]
        x1, x2 = R1 * rho0 / rho, R2 * rho0 / rho
        f = A1 * (1.0 - w / x1) * np.exp(-x1) + A2 * (1.0 - w / x2) * np.exp(-x2) - w * rho * e0
        return np.full_like(rho, w), f
    if kind == EOS["SHOCKWAVE"]:
        rho0, g0, c0, s1, s2, s3, b, e0 = c[:8]
        mu = rho / rho0 - 1.0
        m1 = mu + 1.0
        N = 1.0 + (1.0 - 0.5 * g0) * mu - 0.5 * b * mu * mu
        D = 1.0 - (s1 - 1.0) * mu - s2 * mu * mu / m1 - s3 * mu**3 / (m1 * m1)
        K = rho0 * c0 * c0
        pc = np.where(mu > 0.0, K * mu * N / (D * D), K * mu)
        gr = (g0 + b * mu) * rho0
        return gr / rho, pc - gr * e0
    if kind == EOS["SHOCKWAVE2"]:
        rho0, g0, c0, s, al, e0, p0 = c[:7]
        eta = 1.0 - rho0 / rho
        pH = p0 + rho0 * c0 * c0 * eta / (1.0 - s * eta) ** 2
        eH = e0 + (pH + p0) * eta / (2.0 * rho0)
        G = g0 * (rho0 / rho) ** al
        return G, pH - G * rho * eH
    return np.full_like(rho, params.gamma[k] - 1.0), np.full_like(rho, -params.gamma[k] * params.pinf[k])


def mixture_S_PI(params: HydroParams, a0, ar0, ar1):
    """S and PI of the pressure-equilibrium mixture (p = (rho e - PI)/S)."""
    a0 = np.asarray(a0, dtype=np.float64)
    S = np.zeros(np.broadcast_shapes(a0.shape, np.shape(ar0), np.shape(ar1)))
    PI = np.zeros_like(S)
    for k, (a, ar) in enumerate(((a0, ar0), (1.0 - a0, ar1))):
        rho0 = params.mg[k][0] if params.eos[k] != EOS["STIFFENED"] else 1.0
        rho = np.where(a > 0.0, np.maximum(np.asarray(ar) / np.where(a > 0.0, a, 1.0), params.smallr), rho0)
        G, f = mg_law(params, k, rho)
        xi = 1.0 / G
        S = S + a * xi
        PI = PI - a * xi * f
    return S, PI


def prim_to_cons(dim, params: HydroParams, a0, ar0, ar1, p, vel):
    """Conservative vector [nv, ...] from primitive fields (pressure-equilibrium mixture)."""
    I = ids(dim)
    a0 = np.asarray(a0, dtype=np.float64)
    shape = np.broadcast_shapes(a0.shape, np.shape(ar0), np.shape(ar1), np.shape(p), *[np.shape(v) for v in vel])
    U = np.zeros((I["NV"],) + shape)
    a1 = 1.0 - a0
    if params.eos == (0, 0):
        xi = [1.0 / (g - 1.0) for g in params.gamma]
        gpx = [params.gamma[k] * params.pinf[k] * xi[k] for k in range(2)]
        S = a0 * xi[0] + a1 * xi[1]
        PI = a0 * gpx[0] + a1 * gpx[1]
    else:
        S, PI = mixture_S_PI(params, a0, ar0, ar1)
    rho = ar0 + ar1
    rhoe = p * S + PI
    ek = 0.0
    for v in vel:
        ek = ek + v * v
    U[I["ID"]] = rho
    U[I["IE"]] = rhoe + 0.5 * rho * ek
    U[I["IU"]] = rho * vel[0]
    U[I["IV"]] = rho * vel[1]
    if dim == 3:
        U[I["IW"]] = rho * vel[2]
    U[I["IA0"]] = a0
    U[I["IAD0"]] = ar0
    U[I["IA1"]] = a1
    U[I["IAD1"]] = ar1
    return U


def _alloc_U(table: BlockTable) -> np.ndarray:
    return np.zeros((table.n_total, table.nv, table.ncell), dtype=np.float64)


def rankine_hugoniot(gamma, rho1, p1, mach):
    """Post-shock state of a shock moving at Mach `mach` into gas at rest
    (standard Rankine-Hugoniot relations, as in app/tools/moving_shock.py:79-163)."""
    c1 = math.sqrt(gamma * p1 / rho1)
    m2 = mach * mach
    p2 = p1 * (1.0 + 2.0 * gamma / (gamma + 1.0) * (m2 - 1.0))
    rho2 = rho1 * (gamma + 1.0) * m2 / ((gamma - 1.0) * m2 + 2.0)
    u2 = c1 * 2.0 * (m2 - 1.0) / ((gamma + 1.0) * mach)
    return rho2, p2, u2


# ----------------------------------------------------------------------------
# config 1: 2D gas-water two-fluid shock tube, 512x32 cells, 32x2 blocks of 16^2
# ----------------------------------------------------------------------------
def gas_water_shock_tube(bsize=16, nx_blocks=32, ny_blocks=2, mesh_cls=BlockMesh):
    """Water (stiffened gas 4.4 / 6e8) at x<0.5 against air (ideal 1.4) at x>0.5.

    ``mesh_cls`` (every builder below takes it) is the BlockMesh class that
    holds the forest: a subclass may replace the native forest operations."""
    level = 1
    trees_x = nx_blocks >> level
    trees_y = max(1, ny_blocks >> level)
    mesh = mesh_cls(2, bsize, (trees_x, trees_y), (False, True), level, level, scaling=1.0 / trees_x)
    table = mesh.build()
    params = HydroParams(
        dim=2,
        bsize=bsize,
        gamma=(4.4, 1.4),
        pinf=(6e8, 0.0),
        slope_type=1.0,
        cfl=0.4,
        integrator=INTEGRATOR["HANCOCK"],
        bc=(BC_ZERO_GRADIENT, BC_ZERO_GRADIENT, BC_PERIODIC, BC_PERIODIC, BC_PERIODIC, BC_PERIODIC),
        level_dx=table.level_dx,
    )
    U = _alloc_U(table)
    xc = cell_centers(mesh, table)
    left = xc[:, 0] < 0.5
    eps = 1e-6
    a0 = np.where(left, 1.0 - eps, eps)
    ar0 = a0 * 1000.0
    ar1 = (1.0 - a0) * 50.0
    p = np.where(left, 1e9, 1e5)
    U[: table.n_owned] = np.moveaxis(prim_to_cons(2, params, a0, ar0, ar1, p, (0.0 * p, 0.0 * p)), 0, 1)
    return mesh, table, params, U


# ----------------------------------------------------------------------------
# Mie-Grueneisen two-material shock tubes (the decks' JWL and shock-wave laws)
# ----------------------------------------------------------------------------
MG_LAWS = {
    # LX-17-like detonation products, JWL {rho0, Gamma0, A1, A2, R1, R2, e0}
    "jwl": (EOS["JWL"], (1905.0, 0.8938, 6.321e13, -4.472e9, 11.3, 1.13, 0.0, 0.0)),
    # aluminium, Grueneisen with a cubic Us-up fit {rho0, Gamma0, c0, s1, s2, s3, b, e0}
    "shockwave": (EOS["SHOCKWAVE"], (2700.0, 1.97, 5328.0, 1.4, 0.0, 0.0, 0.48, 0.0)),
    # aluminium, linear Us-up Hugoniot {rho0, Gamma0, c0, s, alpha, e0, p0}
    "shockwave2": (EOS["SHOCKWAVE2"], (2785.0, 2.0, 5328.0, 1.338, 1.0, 0.0, 0.0, 0.0)),
}


def mg_shock_tube(law="jwl", other=None, bsize=16, nx_blocks=16, ny_blocks=2, source_term=0, dim=2):
    """Two-material shock tube with Mie-Grueneisen laws: material 0 (law) at
    x < 0.5 compressed to 1.6 rho0 at high pressure, material 1 (other: a law
    name, or None for the same law, or "air" for an ideal gas) at x > 0.5 at
    rho0 and low pressure.  ZERO_GRADIENT in x, periodic across."""
    level = 1
    trees = [max(1, nx_blocks >> level), max(1, ny_blocks >> level)] + ([max(1, ny_blocks >> level)] if dim == 3 else [])
    per = (False, True) + ((True,) if dim == 3 else ())
    mesh = BlockMesh(dim, bsize, tuple(trees), per, level, level, scaling=1.0 / trees[0])
    table = mesh.build()
    k0, c0 = MG_LAWS[law]
    if other == "air":
        k1, c1, gamma1 = EOS["STIFFENED"], (0.0,) * 8, 1.4
    else:
        k1, c1 = MG_LAWS[other or law]
        gamma1 = 3.0
    params = HydroParams(
        dim=dim,
        bsize=bsize,
        gamma=(3.0, gamma1),
        pinf=(0.0, 0.0),
        slope_type=1.0,
        cfl=0.4,
        integrator=INTEGRATOR["HANCOCK"],
        source_term=source_term,
        bc=(BC_ZERO_GRADIENT, BC_ZERO_GRADIENT) + (BC_PERIODIC,) * 4,
        level_dx=table.level_dx,
        eos=(k0, k1),
        mg=(tuple(c0), tuple(c1)),
    )
    U = _alloc_U(table)
    xc = cell_centers(mesh, table)
    left = xc[:, 0] < 0.5
    eps = 1e-6
    rho0_0 = c0[0]
    rho0_1 = c1[0] if k1 != EOS["STIFFENED"] else 1.0
    a0 = np.where(left, 1.0 - eps, eps)
    ar0 = a0 * 1.6 * rho0_0
    ar1 = (1.0 - a0) * rho0_1
    p = np.where(left, 2e10, 1e5)
    vel = tuple(0.0 * p for _ in range(dim))
    U[: table.n_owned] = np.moveaxis(prim_to_cons(dim, params, a0, ar0, ar1, p, vel), 0, 1)
    return mesh, table, params, U


# ----------------------------------------------------------------------------
# configs 2 / 3: 2D shock-bubble (air-helium, air-R22) on a 3-level block AMR
# ----------------------------------------------------------------------------
def _shock_bubble_prim(params, xc, dxf, bubble_gamma_rho, mach=1.22):
    x, y = xc[:, 0], xc[:, 1]
    eps = 1e-6
    r = np.sqrt((x - 1.0) ** 2 + (y - 0.5) ** 2)
    # alpha_bubble ramps over 2 finest cells around r = 0.25
    phi = 0.5 * (1.0 - np.tanh((r - 0.25) / (2.0 * dxf)))
    a_b = eps + (1.0 - 2.0 * eps) * phi
    a0 = 1.0 - a_b  # material 0 = air
    rho_b = bubble_gamma_rho[1]
    rho2, p2, u2 = rankine_hugoniot(params.gamma[0], 1.0, 1.0, mach)
    post = x < 0.6
    ar0 = np.where(post, a0 * rho2, a0 * 1.0)
    ar1 = np.where(post, (1.0 - a0) * rho_b * rho2, (1.0 - a0) * rho_b)
    p = np.where(post, p2, 1.0)
    u = np.where(post, u2, 0.0)
    return a0, ar0, ar1, p, u


def shock_bubble(bubble="helium", thinc=False, level_min=4, level_max=6, bsize=16, flag_fn=None, slope_type=1.0, initial_level=None, mesh_cls=BlockMesh):
    """Mach 1.22 shock in air hitting a helium (or R22) bubble; domain [0,4]x[0,1].

    The mesh is refined from ``level_min`` by the refine flags evaluated on the
    initial condition (``flag_fn(table, params, U, level_min, level_max) -> int8
    flags``; SIMPLE_GRADIENT on alpha_rho_k, eps_refine 0.1, eps_coarsen
    0.0125), level by level, with 2:1 balance; the mesh then stays fixed.
    ``initial_level`` (optional) first refines the whole domain uniformly to
    that level (a mesh that a dynamic AMR cycle then coarsens and refines).
    """
    gb = {"helium": (1.648, 0.138), "r22": (1.249, 3.1538)}[bubble]
    mesh = mesh_cls(2, bsize, (4, 1), (False, False), level_min, level_max, scaling=1.0)
    for _ in range(level_min, initial_level if initial_level is not None else level_min):
        mesh.refine(list(mesh.leaves))
    params = HydroParams(
        dim=2,
        bsize=bsize,
        gamma=(1.4, gb[0]),
        pinf=(0.0, 0.0),
        slope_type=slope_type,
        cfl=0.4,
        integrator=INTEGRATOR["HANCOCK"],
        thinc=1 if thinc else 0,
        thinc_beta=1.6,
        thinc_eps=1e-3,
        bc=(BC_ZERO_GRADIENT, BC_ZERO_GRADIENT, BC_WALL, BC_WALL, BC_PERIODIC, BC_PERIODIC),
    )
    dxf = mesh.cell_length(level_max)

    def init(table):
        params.level_dx = table.level_dx
        U = _alloc_U(table)
        xc = cell_centers(mesh, table)
        a0, ar0, ar1, p, u = _shock_bubble_prim(params, xc, dxf, gb)
        U[: table.n_owned] = np.moveaxis(prim_to_cons(2, params, a0, ar0, ar1, p, (u, 0.0 * u)), 0, 1)
        return U

    table, U = refine_from_initial_condition(mesh, params, init, flag_fn, level_min, level_max)
    return mesh, table, params, U


def refine_from_initial_condition(mesh, params, init, flag_fn, level_min, level_max):
    """Static AMR: refine by flags on the analytic initial condition, one level
    at a time, then 2:1 balance, until no block asks for refinement."""
    table = mesh.build()
    U = init(table)
    if flag_fn is None:
        return table, U
    for _ in range(level_max - level_min):
        flags = flag_fn(table, params, U, level_min, level_max)
        keys = [
            (int(table.level[n]),) + tuple(int(v) for v in table.coord[n])
            for n in range(table.n_owned)
            if flags[n] == 2
        ]
        if not keys:
            break
        mesh.refine(keys)
        mesh.balance()
        table = mesh.build()
        U = init(table)
    return table, U


# ----------------------------------------------------------------------------
# config 4: batched droplet advection instances
# ----------------------------------------------------------------------------
class SplitMix64:
    """splitmix64 stream (Steele, Lea & Flood 2014); uniform doubles from the top 53 bits."""

    MASK = (1 << 64) - 1

    def __init__(self, seed: int):
        self.state = seed & self.MASK

    def next_u64(self) -> int:
        self.state = (self.state + 0x9E3779B97F4A7C15) & self.MASK
        z = self.state
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & self.MASK
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & self.MASK
        return z ^ (z >> 31)

    def uniform(self, lo=0.0, hi=1.0) -> float:
        return lo + (hi - lo) * ((self.next_u64() >> 11) * (1.0 / (1 << 53)))


def droplet_instances(n_inst=256, sides=(64, 128, 256, 512), bsize=16, seed=0x5EED2026, mesh_cls=BlockMesh):
    """Independent periodic droplet-advection runs of uneven sizes in one table."""
    rng = SplitMix64(seed)
    tables, meshes, Us = [], [], []
    params = HydroParams(
        dim=2,
        bsize=bsize,
        gamma=(4.4, 1.4),
        pinf=(6e8, 0.0),
        slope_type=1.0,
        cfl=0.4,
        integrator=INTEGRATOR["HANCOCK"],
        bc=(BC_PERIODIC,) * 6,
    )
    specs = []
    for _ in range(n_inst):
        side = sides[min(int(rng.uniform() * len(sides)), len(sides) - 1)]
        radius = rng.uniform(0.15, 0.3)
        u = rng.uniform(-1.0, 1.0)
        v = rng.uniform(-1.0, 1.0)
        specs.append((side, radius, u, v))
    for side, radius, u, v in specs:
        # one tree of unit length at level log2(side / bsize)
        level = int(round(math.log2(side // bsize)))
        mesh = mesh_cls(2, bsize, (1, 1), (True, True), level, level, scaling=1.0)
        t = mesh.build()
        # all instances share the level -> dx table of a unit tree
        xc = cell_centers(mesh, t)
        r = np.sqrt((xc[:, 0] - 0.5) ** 2 + (xc[:, 1] - 0.5) ** 2)
        dx = mesh.cell_length(level)
        phi = 0.5 * (1.0 - np.tanh((r - radius) / (2.0 * dx)))
        eps = 1e-6
        a0 = eps + (1.0 - 2.0 * eps) * phi  # material 0 = droplet (water)
        ar0 = a0 * 1000.0
        ar1 = (1.0 - a0) * 1.0
        p = np.full_like(a0, 1e5)
        Ui = np.zeros((t.n_total, t.nv, t.ncell))
        Ui[: t.n_owned] = np.moveaxis(prim_to_cons(2, params, a0, ar0, ar1, p, (u + 0 * p, v + 0 * p)), 0, 1)
        tables.append(t)
        meshes.append(mesh)
        Us.append(Ui)
    table = concat_tables(tables)
    params.level_dx = table.level_dx
    U = np.concatenate([Ui[: t.n_owned] for Ui, t in zip(Us, tables)])
    return meshes, table, params, U, specs


# ----------------------------------------------------------------------------
# config 5: 3D triple point
# ----------------------------------------------------------------------------
def triple_point_3d(level_min=0, level_max=3, bsize=8, nbrick=(14, 6, 3), scaling=0.5, thinc=True, flag_fn=None, mesh_cls=BlockMesh):
    """Three-region triple-point problem on [0,7]x[0,3]x[0,1.5]."""
    mesh = mesh_cls(3, bsize, nbrick, (False, False, False), level_min, level_max, scaling=scaling)
    params = HydroParams(
        dim=3,
        bsize=bsize,
        gamma=(1.5, 1.4),
        pinf=(0.0, 0.0),
        slope_type=1.0,
        cfl=0.4,
        integrator=INTEGRATOR["HANCOCK"],
        thinc=1 if thinc else 0,
        thinc_beta=1.6,
        thinc_eps=1e-3,
        bc=(BC_ZERO_GRADIENT,) * 6,
    )

    def init(table):
        params.level_dx = table.level_dx
        U = _alloc_U(table)
        xc = cell_centers(mesh, table)
        x, y = xc[:, 0], xc[:, 1]
        eps = 1e-6
        left = x < 1.0
        top = (~left) & (y > 1.5)
        a0 = np.where(top, eps, 1.0 - eps)
        rho = np.where(left, 1.0, np.where(top, 0.125, 1.0))
        p = np.where(left, 1.0, 0.1)
        ar0 = a0 * rho
        ar1 = (1.0 - a0) * rho
        z = 0.0 * p
        U[: table.n_owned] = np.moveaxis(prim_to_cons(3, params, a0, ar0, ar1, p, (z, z, z)), 0, 1)
        return U

    table, U = refine_from_initial_condition(mesh, params, init, flag_fn, level_min, level_max)
    return mesh, table, params, U
