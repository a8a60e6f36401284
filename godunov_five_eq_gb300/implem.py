"""Host-side mirror of the reference's GodunovImplemBase over the C ABI.

``GodunovImplemGB300`` keeps the reference's member names and argument
meaning (scheme/GodunovImplemBase.h:59-198, scheme/GodunovImplemV0.h:42-214):

* ``resize_auxiliary_data(table)``   -> g5_set_mesh
* ``total_mem_size_in_bytes()``      -> g5_mem_bytes
* ``do_time_step(U, U2, dt)``        -> g5_step          (U2 <- step(U))
* ``do_time_step(U, U2, t, dt)``     -> same (t is unused, as in V0 for
  every problem but circle_advection)
* ``compute_dt_local(U)``            -> g5_compute_inv_dt, dt = cfl / invDt
  (SolverGodunovFiveEq.cpp:367-390)
* ``fill_outside_quadrants(U)``      -> g5_fill_outside
  (SolverGodunovFiveEq.cpp:977-1019)

Device arrays are torch CUDA tensors of dtype float64 and shape
``[n_blocks, nv, bsize^dim]`` (torch provides device memory and streams
only).  The product path always runs the CUDA library: if it cannot be
loaded, construction raises.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build as _build

G5_MODE_FP64 = 0
G5_MODE_MIXED = 1
MODES = {"fp64": G5_MODE_FP64, "mixed": G5_MODE_MIXED}

ERRORS = {
    -1: "G5_ERR_ARG",
    -2: "G5_ERR_CUDA",
    -3: "G5_ERR_NONPHYSICAL",
    -4: "G5_ERR_TIMEOUT",
    -5: "G5_ERR_MESH",
    -6: "G5_ERR_UNSUPPORTED",
}


class G5Error(RuntimeError):
    def __init__(self, code, what=""):
        super().__init__(f"{what}: {ERRORS.get(code, code)}")
        self.code = code


class G5Params(ctypes.Structure):
    _fields_ = [
        ("dim", ctypes.c_int32),
        ("bsize", ctypes.c_int32),
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


class G5Mesh(ctypes.Structure):
    _fields_ = [
        ("n_owned", ctypes.c_int32),
        ("n_outside", ctypes.c_int32),
        ("n_inst", ctypes.c_int32),
        ("reserved", ctypes.c_int32),
        ("level", ctypes.c_void_p),
        ("coord", ctypes.c_void_p),
        ("nbr", ctypes.c_void_p),
        ("nbr_rel", ctypes.c_void_p),
        ("out_src", ctypes.c_void_p),
        ("out_normal", ctypes.c_void_p),
        ("out_border", ctypes.c_void_p),
        ("inst", ctypes.c_void_p),
    ]


class G5ForestSpec(ctypes.Structure):
    _fields_ = [
        ("dim", ctypes.c_int32),
        ("bsize", ctypes.c_int32),
        ("nbrick", ctypes.c_int32 * 3),
        ("periodic", ctypes.c_int32 * 3),
        ("level_min", ctypes.c_int32),
        ("level_max", ctypes.c_int32),
    ]


class G5Remap(ctypes.Structure):
    _fields_ = [
        ("n_old", ctypes.c_int32),
        ("n_new", ctypes.c_int32),
        ("kind", ctypes.c_void_p),
        ("src", ctypes.c_void_p),
    ]


EXPORTS = [
    "g5_version",
    "g5_create",
    "g5_destroy",
    "g5_set_mesh",
    "g5_mem_bytes",
    "g5_step",
    "g5_step_dev",
    "g5_step_host",
    "g5_step_batched",
    "g5_derived_quantity",
    "g5_pack_fields",
    "g5_compute_inv_dt",
    "g5_fill_outside",
    "g5_begin",
    "g5_advance",
    "g5_run",
    "g5_refine_flags",
    "g5_status",
    "g5_tune",
    "g5_tune_pick",
    "g5_tune_choice",
    "g5_tune_report",
    "g5_set_shape",
    "g5_last_launch_count",
    "g5_step_static",
    "g5_remap",
    "g5_forest_create",
    "g5_forest_destroy",
    "g5_forest_num_leaves",
    "g5_forest_leaves",
    "g5_forest_refine",
    "g5_forest_balance",
    "g5_forest_adapt",
    "g5_forest_table_sizes",
    "g5_forest_table",
]

_lib = None


def library_path() -> str:
    return _build.LIB


def load_library(build_if_missing: bool = True):
    """Load libg5gpu.so (building it in-tree if needed)."""
    global _lib
    if _lib is not None:
        return _lib
    path = library_path()
    if not os.path.exists(path) or not _build.up_to_date():
        if not build_if_missing:
            raise RuntimeError(f"CUDA library missing: {path}")
        _build.build()
    L = ctypes.CDLL(path)
    vp = ctypes.c_void_p
    L.g5_version.restype = ctypes.c_char_p
    L.g5_create.argtypes = [ctypes.POINTER(G5Params), ctypes.POINTER(vp)]
    L.g5_destroy.argtypes = [vp]
    L.g5_set_mesh.argtypes = [vp, ctypes.POINTER(G5Mesh)]
    L.g5_mem_bytes.restype = ctypes.c_int64
    L.g5_mem_bytes.argtypes = [vp]
    L.g5_step.argtypes = [vp, vp, vp, vp, ctypes.c_int, vp, vp]
    L.g5_step_dev.argtypes = [vp, vp, vp, vp, ctypes.c_int, vp, vp]
    L.g5_step_host.argtypes = [vp, vp, vp, vp, ctypes.c_int, vp, vp]
    L.g5_step_batched.argtypes = [vp, vp, vp, vp, ctypes.c_int, vp, ctypes.c_int, vp, vp]
    L.g5_derived_quantity.argtypes = [vp, vp, ctypes.c_int, ctypes.c_int64, ctypes.c_int64, vp, vp]
    L.g5_pack_fields.argtypes = [vp, vp, vp, ctypes.c_int, ctypes.c_int64, ctypes.c_int64, vp, vp]
    L.g5_compute_inv_dt.argtypes = [vp, vp, vp, vp]
    L.g5_fill_outside.argtypes = [vp, vp, vp]
    L.g5_run.argtypes = [vp, vp, vp, ctypes.c_int, ctypes.c_int, vp, vp]
    L.g5_begin.argtypes = [vp, vp, vp]
    L.g5_advance.argtypes = [vp, vp, vp, ctypes.c_int, vp, vp]
    L.g5_refine_flags.argtypes = [vp, vp, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_int, vp, vp]
    L.g5_status.argtypes = [vp, vp]
    L.g5_tune.argtypes = [vp, vp, vp, ctypes.c_int, vp]
    L.g5_tune_pick.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_float]
    L.g5_tune_choice.argtypes = [vp, ctypes.c_int, vp]
    L.g5_tune_report.argtypes = [vp, ctypes.c_int, vp, vp, ctypes.c_int]
    L.g5_set_shape.argtypes = [vp, ctypes.c_int, vp]
    L.g5_last_launch_count.argtypes = [vp]
    L.g5_remap.argtypes = [vp, ctypes.POINTER(G5Remap), vp, vp, vp]
    L.g5_step_static.argtypes = [ctypes.POINTER(G5Params), ctypes.POINTER(G5Mesh), vp, vp, vp, ctypes.c_int, vp, vp, vp]
    L.g5_forest_create.argtypes = [ctypes.POINTER(G5ForestSpec), vp, ctypes.c_int64, ctypes.POINTER(vp)]
    L.g5_forest_destroy.argtypes = [vp]
    L.g5_forest_num_leaves.restype = ctypes.c_int64
    L.g5_forest_num_leaves.argtypes = [vp]
    L.g5_forest_leaves.argtypes = [vp, vp]
    L.g5_forest_refine.argtypes = [vp, vp, ctypes.c_int64]
    L.g5_forest_balance.argtypes = [vp]
    L.g5_forest_adapt.restype = ctypes.c_int64
    L.g5_forest_adapt.argtypes = [vp, vp, ctypes.c_int64, vp, vp, ctypes.c_int64]
    L.g5_forest_table_sizes.argtypes = [vp, ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int32)]
    L.g5_forest_table.argtypes = [vp, vp, vp, vp, vp, vp, vp, vp]
    _lib = L
    return L


def make_params(p) -> G5Params:
    o = G5Params()
    o.dim = p.dim
    o.bsize = p.bsize
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


def _torch():
    import torch

    return torch


def _dptr(t) -> int:
    import torch

    if not isinstance(t, torch.Tensor) or not t.is_cuda or t.dtype != torch.float64 or not t.is_contiguous():
        raise TypeError("expected a contiguous float64 CUDA tensor")
    return t.data_ptr()


def _stream(stream):
    import torch

    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


class GodunovImplemGB300:
    """GB300 implementation of the reference's GodunovImplemBase (implementation_version 3)."""

    implementation_version = 3

    def __init__(self, params, table=None):
        self.lib = load_library()
        self.params = params
        self._prm = make_params(params)
        ctx = ctypes.c_void_p()
        rc = self.lib.g5_create(ctypes.byref(self._prm), ctypes.byref(ctx))
        if rc != 0:
            raise G5Error(rc, "g5_create")
        self.ctx = ctx
        self.table = None
        if table is not None:
            self.resize_auxiliary_data(table)

    def close(self):
        if getattr(self, "ctx", None):
            self.lib.g5_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # --------------------------------------------------------------- the API
    def resize_auxiliary_data(self, table):
        keep = dict(
            level=np.ascontiguousarray(table.level, np.int32),
            coord=np.ascontiguousarray(table.coord, np.int32),
            nbr=np.ascontiguousarray(table.nbr, np.int32),
            nbr_rel=np.ascontiguousarray(table.nbr_rel, np.int8),
            out_src=np.ascontiguousarray(table.out_src, np.int32),
            out_normal=np.ascontiguousarray(table.out_normal, np.int8),
            out_border=np.ascontiguousarray(table.out_border, np.int8),
            inst=np.ascontiguousarray(table.inst, np.int32),
        )
        m = G5Mesh()
        m.n_owned = table.n_owned
        m.n_outside = table.n_outside
        m.n_inst = table.n_inst
        for k, v in keep.items():
            setattr(m, k, v.ctypes.data_as(ctypes.c_void_p) if v.size else None)
        rc = self.lib.g5_set_mesh(self.ctx, ctypes.byref(m))
        if rc != 0:
            raise G5Error(rc, "g5_set_mesh")
        self.table = table

    def total_mem_size_in_bytes(self) -> int:
        return int(self.lib.g5_mem_bytes(self.ctx))

    def do_time_step(self, U, U2, *args, mode="fp64", inv_dt_out=None, stream=None):
        """do_time_step(U, U2, dt) or do_time_step(U, U2, t, dt); dt scalar or per instance."""
        dt = args[-1]
        dt = np.ascontiguousarray(np.broadcast_to(np.asarray(dt, np.float64), (self.table.n_inst,)))
        rc = self.lib.g5_step(
            self.ctx,
            ctypes.c_void_p(_dptr(U)),
            ctypes.c_void_p(_dptr(U2)),
            dt.ctypes.data_as(ctypes.c_void_p),
            MODES[mode],
            ctypes.c_void_p(_dptr(inv_dt_out)) if inv_dt_out is not None else None,
            _stream(stream),
        )
        if rc != 0:
            raise G5Error(rc, "g5_step")

    def do_time_step_dev(self, U, U2, dt_dev, mode="fp64", inv_dt_out=None, stream=None):
        rc = self.lib.g5_step_dev(
            self.ctx,
            ctypes.c_void_p(_dptr(U)),
            ctypes.c_void_p(_dptr(U2)),
            ctypes.c_void_p(_dptr(dt_dev)),
            MODES[mode],
            ctypes.c_void_p(_dptr(inv_dt_out)) if inv_dt_out is not None else None,
            _stream(stream),
        )
        if rc != 0:
            raise G5Error(rc, "g5_step_dev")

    def do_time_step_batched(self, U, U2, dt_dev, instances, mode="fp64", inv_dt_out=None, stream=None):
        """g5_step_batched: one step of the listed instances only (dt_dev[n_inst] on the device)."""
        inst = np.ascontiguousarray(np.asarray(instances, dtype=np.int32).reshape(-1))
        rc = self.lib.g5_step_batched(
            self.ctx,
            ctypes.c_void_p(_dptr(U)),
            ctypes.c_void_p(_dptr(U2)),
            ctypes.c_void_p(_dptr(dt_dev)),
            MODES[mode],
            inst.ctypes.data_as(ctypes.c_void_p),
            int(inst.size),
            ctypes.c_void_p(_dptr(inv_dt_out)) if inv_dt_out is not None else None,
            _stream(stream),
        )
        if rc != 0:
            raise G5Error(rc, "g5_step_batched")

    def do_time_step_host(self, U_host, U2_host, dt, mode="fp64", inv_dt_out=None, stream=None):
        """g5_step_host: U and U2 are CPU tensors (pinned for overlap); the copies
        run chunk by chunk, overlapped with the step.  Asynchronous on `stream`."""
        for T in (U_host, U2_host):
            if T.is_cuda or not T.is_contiguous() or T.dtype != _torch().float64:
                raise ValueError("U_host/U2_host must be contiguous float64 CPU tensors")
        dt = np.ascontiguousarray(np.broadcast_to(np.asarray(dt, np.float64), (self.table.n_inst,)))
        self._dt_keep = dt
        inv = None
        if inv_dt_out is not None:
            if inv_dt_out.is_cuda or inv_dt_out.dtype != _torch().float64:
                raise ValueError("inv_dt_out must be a float64 CPU tensor")
            inv = ctypes.c_void_p(inv_dt_out.data_ptr())
        rc = self.lib.g5_step_host(
            self.ctx,
            ctypes.c_void_p(U_host.data_ptr()),
            ctypes.c_void_p(U2_host.data_ptr()),
            dt.ctypes.data_as(ctypes.c_void_p),
            MODES[mode],
            inv,
            _stream(stream),
        )
        if rc != 0:
            raise G5Error(rc, "g5_step_host")

    DERIVED_QUANTITIES = ("RHO_MIX", "THERMAL_PRESSURE", "SPEED_OF_SOUND", "SPECIFIC_EKIN", "LOCAL_MACH_NUMBER", "VX", "VY", "VZ")

    def derived_quantity(self, U, quantity, oct_begin=0, num_octs=None, out=None, stream=None):
        """g5_derived_quantity (ComputeDerivedQuantities::run): one quantity per cell
        of blocks [oct_begin, oct_begin + num_octs) into out[n_blocks, 1, ncell]."""
        import torch

        q = self.DERIVED_QUANTITIES.index(quantity.upper()) if isinstance(quantity, str) else int(quantity)
        n = self.table.n_total
        num_octs = n - oct_begin if num_octs is None else num_octs
        if out is None:
            out = torch.zeros((n, 1, self.table.ncell), dtype=torch.float64, device=U.device)
        rc = self.lib.g5_derived_quantity(
            self.ctx, ctypes.c_void_p(_dptr(U)), q, int(oct_begin), int(num_octs), ctypes.c_void_p(_dptr(out)), _stream(stream)
        )
        if rc != 0:
            raise G5Error(rc, "g5_derived_quantity")
        return out

    FIELD_DERIVED = 64
    MAX_PACK_FIELDS = 16

    def pack_fields(self, U, fields, oct_begin=0, num_octs=None, out=None, stream=None):
        """g5_pack_fields: the datasets of one output file in one pass over U:
        fields[k] a variable of U (the reference's VarId) or FIELD_DERIVED + a
        derived quantity; returns out[len(fields), num_octs, ncell] (device)."""
        import torch

        fields = [int(f) for f in fields]
        n = self.table.n_owned if num_octs is None else int(num_octs)
        if out is None:
            out = torch.empty((len(fields), n, self.table.ncell), dtype=torch.float64, device=U.device)
        arr = (ctypes.c_int32 * max(len(fields), 1))(*fields)
        rc = self.lib.g5_pack_fields(
            self.ctx, ctypes.c_void_p(_dptr(U)), arr, len(fields), int(oct_begin), n, ctypes.c_void_p(_dptr(out)), _stream(stream)
        )
        if rc != 0:
            raise G5Error(rc, "g5_pack_fields")
        return out

    def compute_inv_dt(self, U, out=None, stream=None):
        import torch

        if out is None:
            out = torch.zeros(self.table.n_inst, dtype=torch.float64, device=U.device)
        rc = self.lib.g5_compute_inv_dt(self.ctx, ctypes.c_void_p(_dptr(U)), ctypes.c_void_p(_dptr(out)), _stream(stream))
        if rc != 0:
            raise G5Error(rc, "g5_compute_inv_dt")
        return out

    def compute_dt_local(self, U, stream=None):
        """dt = cfl / invDt per instance (SolverGodunovFiveEq.cpp:386), as one
        correctly rounded FP64 division (a scalar divided by a tensor would be
        evaluated as scalar x reciprocal, one rounding more)."""
        inv = self.compute_inv_dt(U, stream=stream)
        return inv.new_full(inv.shape, float(self.params.cfl)) / inv

    def fill_outside_quadrants(self, U, stream=None):
        rc = self.lib.g5_fill_outside(self.ctx, ctypes.c_void_p(_dptr(U)), _stream(stream))
        if rc != 0:
            raise G5Error(rc, "g5_fill_outside")

    def run(self, U, U2, nsteps, mode="fp64", dt_hist=None, stream=None):
        """Solver loop: nsteps x {dt = cfl/invDt; step; fill outside}; final state in U."""
        rc = self.lib.g5_run(
            self.ctx,
            ctypes.c_void_p(_dptr(U)),
            ctypes.c_void_p(_dptr(U2)),
            int(nsteps),
            MODES[mode],
            ctypes.c_void_p(_dptr(dt_hist)) if dt_hist is not None else None,
            _stream(stream),
        )
        if rc != 0:
            raise G5Error(rc, "g5_run")

    def begin(self, U, stream=None):
        """g5_begin: fill outside blocks of U and set the CFL accumulator to inv_dt(U)."""
        rc = self.lib.g5_begin(self.ctx, ctypes.c_void_p(_dptr(U)), _stream(stream))
        if rc != 0:
            raise G5Error(rc, "g5_begin")

    def advance(self, U, U2, mode="fp64", dt_out=None, stream=None):
        """g5_advance: one solver step U -> U2 with the device-resident dt (graph replay)."""
        rc = self.lib.g5_advance(
            self.ctx,
            ctypes.c_void_p(_dptr(U)),
            ctypes.c_void_p(_dptr(U2)),
            MODES[mode],
            ctypes.c_void_p(_dptr(dt_out)) if dt_out is not None else None,
            _stream(stream),
        )
        if rc != 0:
            raise G5Error(rc, "g5_advance")

    def refine_flags(self, U, indicator=0, eps_refine=0.1, eps_coarsen=0.0125, eps_lohner=0.02, level_min=0, level_max=30, stream=None):
        import torch

        flags = torch.empty(self.table.n_owned, dtype=torch.int8, device=U.device)
        rc = self.lib.g5_refine_flags(
            self.ctx,
            ctypes.c_void_p(_dptr(U)),
            int(indicator),
            float(eps_refine),
            float(eps_coarsen),
            float(eps_lohner),
            int(level_min),
            int(level_max),
            ctypes.c_void_p(flags.data_ptr()),
            _stream(stream),
        )
        if rc != 0:
            raise G5Error(rc, "g5_refine_flags")
        return flags

    def remap(self, rt, U_old, U_new, stream=None):
        """g5_remap: owned blocks of U_new (the adapted mesh) from U_old, by the
        old -> new map `rt` (mesh.RemapTable) of one adaptation."""
        kind = np.ascontiguousarray(rt.kind, np.int8)
        src = np.ascontiguousarray(rt.src, np.int32)
        r = G5Remap(int(rt.n_old), int(rt.n_new), kind.ctypes.data, src.ctypes.data)
        rc = self.lib.g5_remap(self.ctx, ctypes.byref(r), ctypes.c_void_p(_dptr(U_old)), ctypes.c_void_p(_dptr(U_new)), _stream(stream))
        if rc != 0:
            raise G5Error(rc, "g5_remap")

    def do_amr_cycle(self, mesh, U, indicator=0, eps_refine=0.1, eps_coarsen=0.0125, eps_lohner=0.02, stream=None):
        """SolverGodunovFiveEq::do_amr_cycle (SolverGodunovFiveEq.cpp:258-314) on
        one GPU: boundary fill and refine flags of U on the device, forest
        adaptation on the host (`mesh.adapt`), remap of U to the new mesh on
        the device, block table upload (resize_auxiliary_data) and boundary
        fill of the new state.  Returns (new U, its block table, the remap)."""
        import torch

        self.fill_outside_quadrants(U, stream=stream)
        flags = self.refine_flags(U, indicator, eps_refine, eps_coarsen, eps_lohner, mesh.level_min, mesh.level_max, stream=stream)
        rt = mesh.adapt(flags.cpu().numpy())
        table = mesh.build()
        U_new = torch.empty((table.n_total, table.nv, table.ncell), dtype=torch.float64, device=U.device)
        self.remap(rt, U, U_new, stream=stream)
        self.resize_auxiliary_data(table)
        self.fill_outside_quadrants(U_new, stream=stream)
        return U_new, table, rt

    def status(self, stream=None) -> int:
        rc = self.lib.g5_status(self.ctx, _stream(stream))
        if rc < 0:
            raise G5Error(rc, "g5_status")
        return rc

    def tune(self, U, U2, mode="fp64", stream=None) -> dict:
        """g5_tune: time the candidate launch shapes of `mode` on U -> U2 (U2
        is overwritten) and keep the fastest; returns the chosen shape."""
        rc = self.lib.g5_tune(self.ctx, ctypes.c_void_p(_dptr(U)), ctypes.c_void_p(_dptr(U2)), MODES[mode], _stream(stream))
        if rc < 0:
            raise G5Error(rc, "g5_tune")
        return self.tune_choice(mode)

    # reflux_layout (FP32-bulk 2D reflux pass): 0 eight lanes per deferred
    # cell, 1 one thread per cell, 2 eight lanes per cell in the step
    # kernel's tail
    SHAPE_KEYS = ("ctas_per_sm", "claim", "walk_cf_first", "reflux_layout")

    def tune_choice(self, mode="fp64") -> dict:
        out = (ctypes.c_int32 * 4)()
        rc = self.lib.g5_tune_choice(self.ctx, MODES[mode], out)
        if rc != 0:
            raise G5Error(rc, "g5_tune_choice")
        return dict(zip(self.SHAPE_KEYS, [int(v) for v in out]))

    def tune_report(self, mode="fp64") -> list:
        """[(shape dict, ms per step)] of the last g5_tune of `mode`."""
        n = self.lib.g5_tune_report(self.ctx, MODES[mode], None, None, 0)
        if n < 0:
            raise G5Error(n, "g5_tune_report")
        shapes = (ctypes.c_int32 * max(n, 1))()
        ms = (ctypes.c_float * max(n, 1))()
        self.lib.g5_tune_report(self.ctx, MODES[mode], shapes, ms, n)
        return [(unpack_shape(int(shapes[i])), float(ms[i])) for i in range(n)]

    def set_shape(self, mode="fp64", ctas_per_sm=0, claim=1, walk_cf_first=1, reflux_layout=2):
        arr = (ctypes.c_int32 * 4)(ctas_per_sm, claim, walk_cf_first, reflux_layout)
        rc = self.lib.g5_set_shape(self.ctx, MODES[mode], arr)
        if rc != 0:
            raise G5Error(rc, "g5_set_shape")

    def last_launch_count(self) -> int:
        return int(self.lib.g5_last_launch_count(self.ctx))


def unpack_shape(code: int) -> dict:
    """A packed launch shape of g5_tune (ctas_per_sm + 16 claim + 32 walk + 64 reflux)."""
    return {"ctas_per_sm": code & 15, "claim": (code >> 4) & 1, "walk_cf_first": (code >> 5) & 1, "reflux_layout": (code >> 6) & 3}


def tune_pick(ms, default_index, margin=0.02) -> int:
    """The tuner's selection rule (g5_tune_pick, host only)."""
    lib = load_library()
    arr = (ctypes.c_float * len(ms))(*ms)
    rc = lib.g5_tune_pick(arr, len(ms), int(default_index), float(margin))
    if rc < 0:
        raise G5Error(rc, "g5_tune_pick")
    return rc


def gpu_flag_fn(indicator=0, eps_refine=0.1, eps_coarsen=0.0125, eps_lohner=0.02):
    """Refine-flag callback (runs g5_refine_flags on the GPU) for
    configs.refine_from_initial_condition."""

    def fn(table, params, U, level_min, level_max):
        import torch

        impl = GodunovImplemGB300(params, table)
        d = torch.from_numpy(U).cuda()
        impl.fill_outside_quadrants(d)
        f = impl.refine_flags(d, indicator, eps_refine, eps_coarsen, eps_lohner, level_min, level_max)
        torch.cuda.synchronize()
        out = f.cpu().numpy()
        impl.close()
        return out

    return fn
