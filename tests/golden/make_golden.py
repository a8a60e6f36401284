"""Generate golden vectors for the HLLC solver and the conservative ->
primitive conversion from the reference's own code.

The reference's model code (models/RiemannSolvers.h:57-262, models/utils.h:36-250,
models/HydroSettings.cpp:18-29) is compiled in place from the reference tree
with oracle/refpin (shim headers for the absent Kokkos / kalypsso pieces; the
stiffened-gas mixture EOS is the same restatement as the oracle's).  Seeded
random states cover every HLLC wave configuration (supersonic left/right,
subsonic left/right star states), pure and mixed cells, the density, pressure
and volume-fraction sanitisers.

Run from the repository root (needs the reference tree; writes
tests/golden/hllc_prim_golden.npz):

    python tests/golden/make_golden.py
"""
import ctypes
import os
import subprocess
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
OUT = os.path.join(ROOT, "tests", "golden", "hllc_prim_golden.npz")
PARAM_SETS = np.array(
    [
        [4.4, 1.4, 6e8, 0.0, 1e-10, 1e-10],  # water (stiffened) / air
        [1.4, 1.648, 0.0, 0.0, 1e-10, 1e-10],  # air / helium
        [1.4, 1.249, 0.0, 0.0, 1e-10, 1e-10],  # air / R22
        [1.5, 1.4, 0.0, 0.0, 1e-10, 1e-10],  # triple point
    ]
)


def nv(dim):
    return 8 if dim == 2 else 9


def ids(dim):
    hc = 4 if dim == 2 else 5
    return dict(ID=0, IP=1, IE=1, IU=2, IV=3, IW=4 if dim == 3 else 3, IA0=hc, IAD0=hc + 1, IA1=hc + 2, IAD1=hc + 3)


def rand_alpha(rng, n):
    choices = np.array([0.0, 1.0, 1e-13, 1.0 - 1e-13, 1e-6, 1.0 - 1e-6, 0.5])
    a = rng.uniform(0, 1, n)
    pick = rng.uniform(0, 1, n) < 0.4
    a[pick] = rng.choice(choices, pick.sum())
    return a


def rand_density(rng, n):
    r = 10.0 ** rng.uniform(-6, 3, n)
    pick = rng.uniform(0, 1, n) < 0.1
    r[pick] = rng.choice([0.0, 1e-13, 5e-13], pick.sum())
    return r


def prim_states(rng, n, dim):
    I = ids(dim)
    q = np.zeros((n, nv(dim)))
    q[:, I["IA0"]] = rand_alpha(rng, n)
    q[:, I["IA1"]] = 1 - q[:, I["IA0"]]
    q[:, I["IAD0"]] = rand_density(rng, n) * np.maximum(q[:, I["IA0"]], 1e-6)
    q[:, I["IAD1"]] = rand_density(rng, n) * np.maximum(q[:, I["IA1"]], 1e-6)
    q[:, I["ID"]] = q[:, I["IAD0"]] + q[:, I["IAD1"]]
    q[:, I["IP"]] = 10.0 ** rng.uniform(0, 9.5, n)
    neg = rng.uniform(0, 1, n) < 0.05
    q[neg, I["IP"]] = -rng.uniform(0, 1, neg.sum())
    vel = ["IU", "IV"] + (["IW"] if dim == 3 else [])
    scale = 10.0 ** rng.uniform(-2, 3.7, n)
    for v in vel:
        q[:, I[v]] = rng.normal(0, 1, n) * scale
    return q


def cons_states(rng, n, dim, prm):
    I = ids(dim)
    q = prim_states(rng, n, dim)
    u = q.copy()
    a0 = q[:, I["IA0"]]
    xi = 1.0 / (prm[:2] - 1.0)
    gpx = prm[:2] * prm[2:4] * xi
    S = a0 * xi[0] + (1 - a0) * xi[1]
    PI = a0 * gpx[0] + (1 - a0) * gpx[1]
    rho = q[:, I["ID"]]
    k2 = sum(q[:, I[v]] ** 2 for v in (["IU", "IV"] + (["IW"] if dim == 3 else [])))
    u[:, I["IE"]] = np.abs(q[:, I["IP"]]) * S + PI + 0.5 * rho * k2
    for v in ["IU", "IV"] + (["IW"] if dim == 3 else []):
        u[:, I[v]] = rho * q[:, I[v]]
    # perturbations exercised by the sanitisers: ID != sum of partial densities,
    # alpha slightly outside [0, 1]
    pick = rng.uniform(0, 1, n) < 0.1
    u[pick, I["ID"]] *= 1 + rng.uniform(-1e-3, 1e-3, pick.sum())
    pick = rng.uniform(0, 1, n) < 0.05
    u[pick, I["IA0"]] += rng.choice([-1e-9, 1e-9], pick.sum())
    return u


def main():
    subprocess.run(["make", "-C", os.path.join(ROOT, "oracle", "refpin"), "-s"], check=True)
    lib = ctypes.CDLL(os.path.join(ROOT, "oracle", "_ref", "librefpin.so"))
    vp = ctypes.c_void_p
    lib.ref_hllc.argtypes = [ctypes.c_int, vp, vp, vp, vp]
    lib.ref_prim.restype = ctypes.c_double
    lib.ref_prim.argtypes = [ctypes.c_int, vp, vp, vp]
    rng = np.random.default_rng(0x5EED2026)
    data = {}
    for dim in (2, 3):
        n_per = 300
        I = ids(dim)
        prms, qls, qrs, outs, us, qs, cs = [], [], [], [], [], [], []
        for prm in PARAM_SETS:
            prm = np.ascontiguousarray(prm)
            ql = prim_states(rng, n_per, dim)
            qr = prim_states(rng, n_per, dim)
            out = np.zeros((n_per, nv(dim) + 3))
            for i in range(n_per):
                a, b, o = np.ascontiguousarray(ql[i]), np.ascontiguousarray(qr[i]), np.zeros(nv(dim) + 3)
                lib.ref_hllc(dim, prm.ctypes.data_as(vp), a.ctypes.data_as(vp), b.ctypes.data_as(vp), o.ctypes.data_as(vp))
                out[i] = o
            # riemann_hllc leaves the volume-fraction entries of the flux unset
            out[:, I["IA0"]] = 0.0
            out[:, I["IA1"]] = 0.0
            u = cons_states(rng, n_per, dim, prm)
            q = np.zeros_like(u)
            c = np.zeros(n_per)
            for i in range(n_per):
                a, o = np.ascontiguousarray(u[i]), np.zeros(nv(dim))
                c[i] = lib.ref_prim(dim, prm.ctypes.data_as(vp), a.ctypes.data_as(vp), o.ctypes.data_as(vp))
                q[i] = o
            prms.append(np.repeat(prm[None], n_per, 0))
            qls.append(ql)
            qrs.append(qr)
            outs.append(out)
            us.append(u)
            qs.append(q)
            cs.append(c)
        data[f"d{dim}_prm"] = np.concatenate(prms)
        data[f"d{dim}_ql"] = np.concatenate(qls)
        data[f"d{dim}_qr"] = np.concatenate(qrs)
        data[f"d{dim}_hllc"] = np.concatenate(outs)
        data[f"d{dim}_u"] = np.concatenate(us)
        data[f"d{dim}_q"] = np.concatenate(qs)
        data[f"d{dim}_c"] = np.concatenate(cs)
    np.savez_compressed(OUT, **data)
    print("wrote", OUT, {k: v.shape for k, v in data.items()})


if __name__ == "__main__":
    sys.exit(main())
