"""Generate golden vectors of one whole block timestep from the reference's
own scheme code.

oracle/refpin compiles, in place from the reference tree, the functors of
GodunovImplemV0::do_time_step (scheme/GodunovImplemV0.cpp:85-151): limited
slopes, MUSCL-Hancock and THINC reconstruction with HLLC fluxes and their
dt/dx scaling, the per-direction read-back update with the volume-fraction
source term (ALLAIRE_KOKH and MILLER_PUCKETT), the volume-fraction
renormalisation and the CFL reduction, and runs them serially on a periodic
tile of same-level blocks (refpin_scheme_step).  This script stores the
inputs and the reference's outputs for a few parameter sets, 2D and 3D, in
tests/golden/scheme_step_golden.npz, so that the oracle can be checked against
them where the reference tree is absent.

Run from the repository root (needs the reference tree and a built oracle):

    python tests/golden/make_scheme_golden.py           # block steps
    python tests/golden/make_scheme_golden.py --flags   # refinement flags
    python tests/golden/make_scheme_golden.py --fill    # boundary fill
"""
import ctypes
import os
import subprocess
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
OUT = os.path.join(ROOT, "tests", "golden", "scheme_step_golden.npz")
LIB = os.path.join(ROOT, "oracle", "_ref", "librefpin.so")

# name: dim, b, nb (blocks per tile edge), materials, thinc, integrator
# (0 HANCOCK, 1 RK1), source term (0 ALLAIRE_KOKH, 1 MILLER_PUCKETT), slope type, seed
CASES = {
    "2d_muscl_hancock_ak_minmod_water_air": (2, 8, 2, "water_air", 0, 0, 0, 1.0, 1),
    "2d_thinc_hancock_ak_mc_water_air": (2, 8, 2, "water_air", 1, 0, 0, 2.0, 2),
    "2d_muscl_rk1_mp_minmod_water_air": (2, 8, 2, "water_air", 0, 1, 1, 1.0, 3),
    "2d_thinc_hancock_mp_minmod_air_helium": (2, 8, 2, "air_helium", 1, 0, 1, 1.0, 4),
    "3d_muscl_hancock_ak_minmod_water_air": (3, 8, 1, "water_air", 0, 0, 0, 1.0, 5),
    "3d_thinc_hancock_mp_mc_air_r22": (3, 8, 1, "air_r22", 1, 0, 1, 2.0, 6),
}
MATERIALS = {"water_air": ((4.4, 1.4), (6e8, 0.0)), "air_helium": ((1.4, 1.648), (0.0, 0.0)), "air_r22": ((1.4, 1.249), (0.0, 0.0))}


def tile_case(dim, b, nb, materials, thinc, integrator, source_term, slope_type, seed):
    """Mesh, parameters and state of a periodic tile of nb^dim level-0 blocks:
    smooth velocity and pressure fields and a material interface about one
    cell wide (THINC reconstructs there)."""
    from godunov_five_eq_gb300 import configs
    from godunov_five_eq_gb300.mesh import BlockMesh

    gamma, pinf = MATERIALS[materials]
    mesh = BlockMesh(dim, b, (nb,) * dim, (True,) * dim, 0, 0, scaling=1.0)
    t = mesh.build()
    p = configs.HydroParams(
        dim=dim,
        bsize=b,
        gamma=gamma,
        pinf=pinf,
        slope_type=slope_type,
        cfl=0.4,
        integrator=integrator,
        thinc=thinc,
        thinc_beta=1.6,
        thinc_eps=1e-3,
        source_term=source_term,
        bc=(1,) * 6,
        level_dx=t.level_dx,
    )
    rng = np.random.default_rng(seed)
    xc = configs.cell_centers(mesh, t)
    x, y = xc[:, 0], xc[:, 1]
    z = xc[:, 2] if dim == 3 else 0.0 * x
    L = float(nb)
    c0 = rng.uniform(0.3, 0.7, 3) * L
    r = np.sqrt((x - c0[0]) ** 2 + (y - c0[1]) ** 2 + ((z - c0[2]) ** 2 if dim == 3 else 0.0))
    dx = 1.0 / b
    a0 = 1e-6 + (1 - 2e-6) * 0.5 * (1 - np.tanh((r - 0.3 * L) / (0.8 * dx)))
    rho0, rho1 = (1000.0, 1.2) if materials == "water_air" else (1.0, 0.138 if materials == "air_helium" else 3.15)
    k = rng.uniform(0.5, 1.5, 4)
    ar0 = a0 * rho0 * (1 + 0.05 * np.sin(2 * np.pi * k[0] * y / L))
    ar1 = (1 - a0) * rho1 * (1 + 0.05 * np.cos(2 * np.pi * k[1] * x / L))
    pbase = 1e5 if materials == "water_air" else 1.0
    pr = pbase * (1 + 0.3 * np.sin(2 * np.pi * (x + y) / L) + 0.5 * (x < 0.5 * L))
    s = 10.0 if materials == "water_air" else 0.3
    vel = [s * np.cos(2 * np.pi * k[2] * y / L), -0.5 * s * np.sin(2 * np.pi * k[3] * x / L)]
    if dim == 3:
        vel.append(0.3 * s * np.cos(2 * np.pi * z / L))
    U = np.zeros((t.n_total, t.nv, t.ncell))
    U[: t.n_owned] = np.moveaxis(configs.prim_to_cons(dim, p, a0, ar0, ar1, pr, tuple(vel)), 0, 1)
    return mesh, t, p, U


def params_vector(p, thinc, integrator, source_term):
    return np.array(
        [p.gamma[0], p.gamma[1], p.pinf[0], p.pinf[1], p.smallr, p.smallc, p.slope_type, thinc, p.thinc_beta, p.thinc_eps, integrator, source_term],
        dtype=np.float64,
    )


def reference_step(lib, dim, b, nb, prm, U, dt):
    vp = ctypes.c_void_p
    U = np.ascontiguousarray(U, np.float64)
    out = np.zeros_like(U)
    inv = np.zeros(1)
    rc = lib.refpin_scheme_step(prm.ctypes.data_as(vp), dim, b, nb, 0, U.ctypes.data_as(vp), float(dt), out.ctypes.data_as(vp), inv.ctypes.data_as(vp))
    if rc != 0:
        raise RuntimeError(f"refpin_scheme_step failed ({rc})")
    return out, float(inv[0])


def load():
    lib = ctypes.CDLL(LIB)
    vp = ctypes.c_void_p
    lib.refpin_scheme_step.restype = ctypes.c_int
    lib.refpin_scheme_step.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, vp, ctypes.c_double, vp, vp]
    return lib


def main():
    subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "-s"], check=True)
    subprocess.run(["make", "-C", os.path.join(ROOT, "oracle", "refpin"), "-s", "-j8"], check=True)
    lib = load()
    data = {}
    for name, (dim, b, nb, mats, thinc, integ, st, slope, seed) in CASES.items():
        mesh, t, p, U = tile_case(dim, b, nb, mats, thinc, integ, st, slope, seed)
        # dt from the CFL condition of the initial state, written with the case
        from oracle.oracle import Oracle

        o = Oracle(t, p)
        dt = float(o.dt(U)[0])
        o.close()
        prm = params_vector(p, thinc, integ, st)
        out, inv = reference_step(lib, dim, b, nb, prm, U[: t.n_owned], dt)
        data[f"{name}/prm"] = prm
        data[f"{name}/shape"] = np.array([dim, b, nb])
        data[f"{name}/dt"] = np.array([dt])
        data[f"{name}/U"] = U[: t.n_owned]
        data[f"{name}/U2"] = out
        data[f"{name}/inv_dt"] = np.array([inv])
    np.savez_compressed(OUT, **data)
    print("wrote", OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__" and "--flags" not in sys.argv and "--fill" not in sys.argv:
    sys.exit(main())


# ---------------------------------------------------------------------------
# Refinement flags (ComputeRefineFlags::run, scheme/ComputeRefineFlags.cpp:18-368)
# of the reference's own code on periodic tiles of same-level blocks
# (refpin_refine_flags), swept over the thresholds so that each block's
# largest indicator is pinned to an interval: tests/golden/refine_flags_golden.npz
# ---------------------------------------------------------------------------
FLAG_OUT = os.path.join(ROOT, "tests", "golden", "refine_flags_golden.npz")
EPS_REFINE = (0.005, 0.01, 0.02, 0.05, 0.1, 0.2, 0.4, 0.7, 0.95)
EPS_COARSEN = (0.001, 0.003, 0.0125, 0.05, 0.2)
EPS_LOHNER = (0.01, 0.02, 0.1)


def flag_tile(dim, seed):
    """A tile of 4x4 (2D) or 2x2x2 (3D) level-0 blocks of 8^dim cells with a
    material interface over part of it and smooth fields elsewhere."""
    nb = 4 if dim == 2 else 2
    return tile_case(dim, 8, nb, "water_air" if seed % 2 else "air_helium", 0, 0, 0, 1.0, seed), nb


def reference_flags(lib, dim, b, nb, U, indicator, eps_lohner, eps_refine, eps_coarsen, lmin, lmax):
    vp = ctypes.c_void_p
    U = np.ascontiguousarray(U, np.float64)
    nblocks = nb**dim
    out = np.zeros(nblocks, np.int8)
    rc = lib.refpin_refine_flags(dim, b, nb, 0, U.ctypes.data_as(vp), indicator, eps_lohner, eps_refine, eps_coarsen, lmin, lmax, out.ctypes.data_as(vp))
    if rc != 0:
        raise RuntimeError(f"refpin_refine_flags failed ({rc})")
    return out


def load_flags():
    lib = load()
    vp = ctypes.c_void_p
    lib.refpin_refine_flags.restype = ctypes.c_int
    lib.refpin_refine_flags.argtypes = [ctypes.c_int] * 4 + [vp, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_int, vp]
    return lib


def sweep(lib, dim, nb, U):
    """flags[indicator, lohner eps, refine eps, coarsen eps, block] with level 0,
    level_min -1 (coarsening allowed) and level_max 2."""
    out = np.zeros((3, len(EPS_LOHNER), len(EPS_REFINE), len(EPS_COARSEN), nb**dim), np.int8)
    for ind in range(3):
        for a, el in enumerate(EPS_LOHNER):
            for i, er in enumerate(EPS_REFINE):
                for j, ec in enumerate(EPS_COARSEN):
                    out[ind, a, i, j] = reference_flags(lib, dim, 8, nb, U, ind, el, er, ec, -1, 2)
    return out


def main_flags():
    lib = load_flags()
    data = {}
    for seed in (11, 12):
        (mesh, t, p, U), nb = flag_tile(2, seed)
        data[f"seed{seed}/U"] = U[: t.n_owned]
        data[f"seed{seed}/flags"] = sweep(lib, 2, nb, U[: t.n_owned])
    np.savez_compressed(FLAG_OUT, **data)
    print("wrote", FLAG_OUT, os.path.getsize(FLAG_OUT), "bytes")


if __name__ == "__main__" and "--flags" in sys.argv:
    main_flags()


# ---------------------------------------------------------------------------
# Boundary fill (FillOutsideCellFunctor::apply, border_conditions/FillOutside.cpp:
# 44-172) of the reference's own code on non-periodic AMR meshes with
# ZERO_GRADIENT and WALL faces (refpin_fill_outside):
# tests/golden/fill_outside_golden.npz
# ---------------------------------------------------------------------------
FILL_OUT = os.path.join(ROOT, "tests", "golden", "fill_outside_golden.npz")
ZG, WALL = 2, 3
# name: dim, seed, border condition of each face (xmin xmax ymin ymax zmin zmax)
FILL_CASES = {
    "2d_zero_gradient": (2, 1, (ZG,) * 6),
    "2d_wall": (2, 2, (WALL,) * 6),
    "2d_mixed": (2, 3, (ZG, WALL, WALL, ZG, ZG, ZG)),
    "3d_mixed": (3, 4, (WALL, ZG, ZG, WALL, WALL, ZG)),
}


def fill_case(dim, seed):
    """A non-periodic 2:1-balanced AMR mesh (outside quadrants on every face)
    and a state whose every owned value is distinct (1 + its flat index), so
    that each filled value names the value it was copied from."""
    from tests.helpers import amr_mesh

    if dim == 2:
        mesh, t = amr_mesh(dim=2, b=8, nref=3, seed=seed, periodic=False)
    else:
        mesh, t = amr_mesh(dim=3, b=8, nref=2, seed=seed, periodic=False, nbrick=(2, 1, 1), lmin=1, lmax=2)
    U = np.zeros((t.n_total, t.nv, t.ncell))
    U[: t.n_owned] = 1.0 + np.arange(t.n_owned * t.nv * t.ncell, dtype=np.float64).reshape(t.n_owned, t.nv, t.ncell)
    return mesh, t, U


def load_fill():
    lib = load()
    vp = ctypes.c_void_p
    lib.refpin_fill_outside.restype = ctypes.c_int
    lib.refpin_fill_outside.argtypes = [ctypes.c_int] * 4 + [vp] * 5
    return lib


def reference_fill(lib, t, U, bc):
    vp = ctypes.c_void_p
    U = np.ascontiguousarray(U, np.float64).copy()
    src = np.ascontiguousarray(t.out_src, np.int32)
    nrm = np.ascontiguousarray(t.out_normal, np.int8)
    brd = np.ascontiguousarray(t.out_border, np.int8)
    bca = np.ascontiguousarray(bc, np.int32)
    rc = lib.refpin_fill_outside(t.dim, t.bsize, t.n_owned, t.n_outside, src.ctypes.data_as(vp), nrm.ctypes.data_as(vp),
                                 brd.ctypes.data_as(vp), bca.ctypes.data_as(vp), U.ctypes.data_as(vp))
    if rc != 0:
        raise RuntimeError(f"refpin_fill_outside failed ({rc})")
    return U


def main_fill():
    lib = load_fill()
    data = {}
    for name, (dim, seed, bc) in FILL_CASES.items():
        mesh, t, U = fill_case(dim, seed)
        ref = reference_fill(lib, t, U, bc)
        out = ref[t.n_owned :]
        assert np.array_equal(out, np.rint(out)) and np.abs(out).max() < 2**31
        data[f"{name}/outside"] = out.astype(np.int32)  # exact: the values are integers
    np.savez_compressed(FILL_OUT, **data)
    print("wrote", FILL_OUT, os.path.getsize(FILL_OUT), "bytes")


if __name__ == "__main__" and "--fill" in sys.argv:
    main_fill()
