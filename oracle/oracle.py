"""ctypes binding of the CPU oracle (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module; it is the checker, never the measured or shipped path.
Parity status: the scheme arithmetic is pinned to the reference's own code
(HLLC and primitive conversion per state, whole block steps of same-level
tiles through the reference's scheme functors, the refinement flags and the
boundary fill: tests/test_golden.py);
the AMR stencils (restriction, prolongation, coarse/fine face sums), the
mixture EOS and the Youngs normal are restatements of the external core
(see g5_oracle.cpp).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libg5oracle.so")


def build(force: bool = False) -> str:
    src = os.path.join(HERE, "g5_oracle.cpp")
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
        subprocess.run(["make", "-C", HERE, "-s"], check=True)
    return LIB_PATH


class G5OParams(ctypes.Structure):
    _fields_ = [
        ("dim", ctypes.c_int32),
        ("b", ctypes.c_int32),
        ("integrator", ctypes.c_int32),
        ("thinc", ctypes.c_int32),
        ("source_term", ctypes.c_int32),
        ("prolongation", ctypes.c_int32),
        ("bc", ctypes.c_int32 * 6),
        ("gamma", ctypes.c_double * 2),
        ("pinf", ctypes.c_double * 2),
        ("smallr", ctypes.c_double),
        ("smallc", ctypes.c_double),
        ("slope_type", ctypes.c_double),
        ("cfl", ctypes.c_double),
        ("thinc_beta", ctypes.c_double),
        ("thinc_eps", ctypes.c_double),
        ("level_dx", ctypes.c_double * 32),
        ("eos", ctypes.c_int32 * 2),
        ("mg", (ctypes.c_double * 8) * 2),
    ]


class G5OMesh(ctypes.Structure):
    _fields_ = [
        ("n_owned", ctypes.c_int32),
        ("n_outside", ctypes.c_int32),
        ("n_inst", ctypes.c_int32),
        ("pad", ctypes.c_int32),
        ("level", ctypes.c_void_p),
        ("coord", ctypes.c_void_p),
        ("nbr", ctypes.c_void_p),
        ("nbr_rel", ctypes.c_void_p),
        ("out_src", ctypes.c_void_p),
        ("out_normal", ctypes.c_void_p),
        ("out_border", ctypes.c_void_p),
        ("inst", ctypes.c_void_p),
    ]


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        vp, dp = ctypes.c_void_p, ctypes.POINTER(ctypes.c_double)
        L.g5o_create.restype = vp
        L.g5o_create.argtypes = [ctypes.POINTER(G5OMesh), ctypes.POINTER(G5OParams), ctypes.c_int]
        L.g5o_destroy.argtypes = [vp]
        L.g5o_step.argtypes = [vp, vp, vp, vp]
        L.g5o_inv_dt.argtypes = [vp, vp, vp]
        L.g5o_fill_outside.argtypes = [vp, vp]
        L.g5o_ghost_state.argtypes = [vp, vp, ctypes.c_int, vp, vp]
        L.g5o_refine_flags.argtypes = [vp, vp, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_int, vp]
        L.g5o_compute_primitives.restype = ctypes.c_double
        L.g5o_compute_primitives.argtypes = [ctypes.POINTER(G5OParams), vp, vp]
        L.g5o_riemann_hllc.argtypes = [ctypes.POINTER(G5OParams), vp, vp, vp]
        L.g5o_slope.restype = ctypes.c_double
        L.g5o_slope.argtypes = [ctypes.POINTER(G5OParams), ctypes.c_double, ctypes.c_double, ctypes.c_double]
        L.g5o_tanh.restype = ctypes.c_double
        L.g5o_tanh.argtypes = [ctypes.c_double]
        L.g5o_mixture_pressure.restype = ctypes.c_double
        L.g5o_mixture_pressure.argtypes = [ctypes.POINTER(G5OParams)] + [ctypes.c_double] * 5
        L.g5o_mixture_sound_speed.restype = ctypes.c_double
        L.g5o_mixture_sound_speed.argtypes = [ctypes.POINTER(G5OParams)] + [ctypes.c_double] * 5
        L.g5o_remap.argtypes = [ctypes.POINTER(G5OParams), ctypes.c_int, vp, vp, vp, vp]
        L.g5o_remap_mesh.argtypes = [vp, ctypes.c_int, vp, vp, vp, vp]
        L.g5o_derived.argtypes = [ctypes.POINTER(G5OParams), vp, ctypes.c_int, ctypes.c_longlong, ctypes.c_longlong, vp]
        _lib = L
    return _lib


def make_params(p) -> G5OParams:
    """From a godunov_five_eq_gb300.configs.HydroParams-like object."""
    o = G5OParams()
    o.dim = p.dim
    o.b = p.bsize
    o.integrator = p.integrator
    o.thinc = p.thinc
    o.source_term = p.source_term
    o.prolongation = p.prolongation
    for i in range(6):
        o.bc[i] = int(p.bc[i])
    for k in range(2):
        o.gamma[k] = p.gamma[k]
        o.pinf[k] = p.pinf[k]
    o.smallr = p.smallr
    o.smallc = p.smallc
    o.slope_type = p.slope_type
    o.cfl = p.cfl
    o.thinc_beta = p.thinc_beta
    o.thinc_eps = p.thinc_eps
    for i in range(32):
        o.level_dx[i] = float(p.level_dx[i])
    for k in range(2):
        o.eos[k] = int(p.eos[k])
        for j in range(8):
            o.mg[k][j] = float(p.mg[k][j]) if j < len(p.mg[k]) else 0.0
    return o


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


class Oracle:
    """One oracle context per (mesh, params)."""

    def __init__(self, table, params, nthreads: int = 0):
        self.table = table
        self.params = params
        self._keep = dict(
            level=np.ascontiguousarray(table.level, np.int32),
            coord=np.ascontiguousarray(table.coord, np.int32),
            nbr=np.ascontiguousarray(table.nbr, np.int32),
            nbr_rel=np.ascontiguousarray(table.nbr_rel, np.int8),
            out_src=np.ascontiguousarray(table.out_src, np.int32),
            out_normal=np.ascontiguousarray(table.out_normal, np.int8),
            out_border=np.ascontiguousarray(table.out_border, np.int8),
            inst=np.ascontiguousarray(table.inst, np.int32),
        )
        m = G5OMesh()
        m.n_owned = table.n_owned
        m.n_outside = table.n_outside
        m.n_inst = table.n_inst
        for k, v in self._keep.items():
            setattr(m, k, _ptr(v))
        self._mesh = m
        self._prm = make_params(params)
        self.ctx = lib().g5o_create(ctypes.byref(m), ctypes.byref(self._prm), int(nthreads))
        if not self.ctx:
            raise RuntimeError("g5o_create failed")

    def close(self):
        if self.ctx:
            lib().g5o_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def fill_outside(self, U: np.ndarray) -> None:
        assert U.dtype == np.float64 and U.flags.c_contiguous
        lib().g5o_fill_outside(self.ctx, _ptr(U))

    def ghost_state(self, U: np.ndarray, n: int, g) -> np.ndarray:
        """Conservative state the ghost fill of owned block n gives its
        ghosted cell g (block cell coordinates, -2 .. b+1)."""
        assert U.dtype == np.float64 and U.flags.c_contiguous
        gg = np.zeros(3, np.int32)
        gg[: len(g)] = g
        out = np.zeros(self.table.nv)
        if lib().g5o_ghost_state(self.ctx, _ptr(U), int(n), _ptr(gg), _ptr(out)) != 0:
            raise ValueError("ghost cell out of range")
        return out

    def remap(self, rt, U_old: np.ndarray, n_total_new: int) -> np.ndarray:
        """Owned blocks of the adapted mesh from the old state, this context's
        mesh being the old one: as the module-level remap, and under a
        prolongation other than SIMPLE_COPY the refined blocks prolonged over
        the old mesh (U_old's outside blocks filled)."""
        nv = 8 if rt.dim == 2 else 9
        U_old = np.ascontiguousarray(U_old, np.float64)
        U_new = np.zeros((n_total_new, nv, rt.bsize**rt.dim))
        kind = np.ascontiguousarray(rt.kind, np.int8)
        src = np.ascontiguousarray(rt.src, np.int32)
        if lib().g5o_remap_mesh(self.ctx, rt.n_new, _ptr(kind), _ptr(src), _ptr(U_old), _ptr(U_new)) != 0:
            raise ValueError("remap map does not match the context's mesh")
        return U_new

    def inv_dt(self, U: np.ndarray) -> np.ndarray:
        out = np.zeros(self.table.n_inst)
        lib().g5o_inv_dt(self.ctx, _ptr(U), _ptr(out))
        return out

    def dt(self, U: np.ndarray) -> np.ndarray:
        return self.params.cfl / self.inv_dt(U)

    def step(self, U: np.ndarray, dt) -> np.ndarray:
        """One do_time_step: returns U2 (owned blocks updated, outside blocks copied from U)."""
        assert U.dtype == np.float64 and U.flags.c_contiguous
        dt = np.ascontiguousarray(np.broadcast_to(np.asarray(dt, np.float64), (self.table.n_inst,)))
        U2 = U.copy()
        lib().g5o_step(self.ctx, _ptr(U), _ptr(U2), _ptr(dt))
        return U2

    def refine_flags(self, U, indicator=0, eps_refine=0.1, eps_coarsen=0.0125, eps_lohner=0.02, level_min=0, level_max=30):
        flags = np.zeros(self.table.n_owned, np.int8)
        lib().g5o_refine_flags(self.ctx, _ptr(U), int(indicator), eps_refine, eps_coarsen, eps_lohner, level_min, level_max, _ptr(flags))
        return flags

    def run(self, U: np.ndarray, nsteps: int, fill_first: bool = True):
        """Solver loop of SolverGodunovFiveEq::godunov_unsplit (SolverGodunovFiveEq.cpp:480-526).

        HANCOCK / RK1: fill outside, dt, one step.  RK2_SSP (integrator 2): two
        steps without the Hancock predictor and U^{n+1} = 0.5 U^n + 0.5 U2 on
        the owned blocks (the external LinearCombination with the standard
        SSP-RK2 coefficients; its stage-1 combination is the identity)."""
        U = U.copy()
        n = self.table.n_owned
        dts = []
        for _ in range(nsteps):
            self.fill_outside(U)
            dt = self.dt(U)
            dts.append(dt)
            if self.params.integrator == 2:
                R = self.step(U, dt)
                self.fill_outside(R)
                U2 = self.step(R, dt)
                U2[:n] = 0.5 * U[:n] + 0.5 * U2[:n]
                U = U2
            else:
                U = self.step(U, dt)
        self.fill_outside(U)
        return U, np.array(dts)


def remap(params, rt, U_old: np.ndarray, n_total_new: int) -> np.ndarray:
    """Owned blocks of the adapted mesh from the old state (outside blocks left
    zero: fill them with Oracle.fill_outside on the new mesh)."""
    nv = 8 if rt.dim == 2 else 9
    nc = rt.bsize**rt.dim
    U_old = np.ascontiguousarray(U_old, np.float64)
    assert U_old.shape[0] >= rt.n_old
    U_new = np.zeros((n_total_new, nv, nc))
    kind = np.ascontiguousarray(rt.kind, np.int8)
    src = np.ascontiguousarray(rt.src, np.int32)
    prm = make_params(params)
    lib().g5o_remap(ctypes.byref(prm), rt.n_new, _ptr(kind), _ptr(src), _ptr(U_old), _ptr(U_new))
    return U_new


DERIVED_QUANTITIES = ("RHO_MIX", "THERMAL_PRESSURE", "SPEED_OF_SOUND", "SPECIFIC_EKIN", "LOCAL_MACH_NUMBER", "VX", "VY", "VZ")


def derived(params, U: np.ndarray, quantity, begin=0, count=None) -> np.ndarray:
    """ComputeDerivedQuantities on the CPU: out[n_blocks, 1, ncell] (zeros outside the range)."""
    q = DERIVED_QUANTITIES.index(quantity.upper()) if isinstance(quantity, str) else int(quantity)
    U = np.ascontiguousarray(U, np.float64)
    n = U.shape[0]
    count = n - begin if count is None else count
    out = np.zeros((n, 1, U.shape[2]))
    prm = make_params(params)
    lib().g5o_derived(ctypes.byref(prm), _ptr(U), q, int(begin), int(count), _ptr(out))
    return out


def oracle_flag_fn(indicator=0, eps_refine=0.1, eps_coarsen=0.0125, eps_lohner=0.02):
    """Refine-flag callback for configs.refine_from_initial_condition (tests only)."""

    def fn(table, params, U, level_min, level_max):
        o = Oracle(table, params)
        o.fill_outside(U)
        f = o.refine_flags(U, indicator, eps_refine, eps_coarsen, eps_lohner, level_min, level_max)
        o.close()
        return f

    return fn
