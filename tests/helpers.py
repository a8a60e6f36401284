"""Shared helpers of the test suite (small meshes, random smooth states)."""
import numpy as np

from godunov_five_eq_gb300 import configs
from godunov_five_eq_gb300.mesh import BC_PERIODIC, BC_WALL, BC_ZERO_GRADIENT, BlockMesh


def amr_mesh(dim=2, b=8, periodic=True, seed=0, nbrick=(2, 2, 2), lmin=1, lmax=3, nref=3):
    """A small 2:1-balanced AMR forest refined at pseudo-random blocks."""
    mesh = BlockMesh(dim, b, nbrick[:dim], (periodic,) * dim, lmin, lmax)
    rng = np.random.default_rng(seed)
    for _ in range(lmax - lmin):
        leaves = sorted(mesh.leaves)
        pick = rng.choice(len(leaves), size=min(nref, len(leaves)), replace=False)
        mesh.refine([leaves[i] for i in pick])
        mesh.balance()
    return mesh, mesh.build()


def smooth_state(mesh, table, params, seed=0, interface=True):
    """Smooth two-material state (alpha in (0,1) with a sharp-ish interface)."""
    dim = table.dim
    rng = np.random.default_rng(seed)
    xc = configs.cell_centers(mesh, table)
    x = xc[:, 0]
    y = xc[:, 1]
    z = xc[:, 2] if dim == 3 else 0.0 * x
    k = rng.uniform(0.5, 1.5, size=6)
    if interface:
        r = np.sqrt((x - 0.8) ** 2 + (y - 0.9) ** 2 + ((z - 0.7) ** 2 if dim == 3 else 0.0))
        a0 = 1e-6 + (1 - 2e-6) * 0.5 * (1 - np.tanh((r - 0.4) / 0.05))
    else:
        a0 = 0.5 + 0.4 * np.sin(2 * np.pi * k[0] * x) * np.cos(2 * np.pi * y)
    ar0 = a0 * (1000.0 + 10 * np.sin(2 * np.pi * y))
    ar1 = (1 - a0) * (1.2 + 0.1 * np.cos(2 * np.pi * x))
    p = 1e5 * (1 + 0.2 * np.sin(2 * np.pi * (x + y)))
    vel = [10 * np.cos(2 * np.pi * y), -5 * np.sin(2 * np.pi * x)]
    if dim == 3:
        vel.append(3 * np.cos(2 * np.pi * z))
    U = np.zeros((table.n_total, table.nv, table.ncell))
    U[: table.n_owned] = np.moveaxis(configs.prim_to_cons(dim, params, a0, ar0, ar1, p, tuple(vel)), 0, 1)
    return U


def water_air_params(table, dim=2, b=8, bc=None, **kw):
    p = configs.HydroParams(
        dim=dim,
        bsize=b,
        gamma=(4.4, 1.4),
        pinf=(6e8, 0.0),
        slope_type=kw.pop("slope_type", 1.0),
        cfl=0.4,
        bc=bc if bc is not None else (BC_PERIODIC,) * 6,
        level_dx=table.level_dx,
        **kw,
    )
    return p


__all__ = ["amr_mesh", "smooth_state", "water_air_params", "BC_PERIODIC", "BC_WALL", "BC_ZERO_GRADIENT"]
