"""g5_step_static, the allocation-free step, against g5_step.

g5_step_static serves callers that must not allocate device memory while
they advance the solution (a solver whose device memory belongs to its
framework's pool allocator, or a plugin whose host process accounts for every
device allocation).  It runs the same kernels as g5_step with all scratch in
a fixed file-scope device array, so its results must equal g5_step's bit for
bit, in FP64 and in mixed mode, on two consecutive steps (the second call
reuses the array the first one filled).  The mesh has coarse/fine faces, so
the face-record scratch is exercised too.

This file is collected last so that a run stopping at the first failure has
already run every other test; it also passes alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from godunov_five_eq_gb300 import implem  # noqa: E402
from godunov_five_eq_gb300.implem import GodunovImplemGB300  # noqa: E402
from tests.helpers import amr_mesh, smooth_state, water_air_params  # noqa: E402

pytestmark = pytest.mark.gpu


def _host_mesh(t):
    keep = dict(
        level=np.ascontiguousarray(t.level, np.int32),
        coord=np.ascontiguousarray(t.coord, np.int32),
        nbr=np.ascontiguousarray(t.nbr, np.int32),
        nbr_rel=np.ascontiguousarray(t.nbr_rel, np.int8),
        out_src=np.ascontiguousarray(t.out_src, np.int32),
        out_normal=np.ascontiguousarray(t.out_normal, np.int8),
        out_border=np.ascontiguousarray(t.out_border, np.int8),
        inst=np.ascontiguousarray(t.inst, np.int32),
    )
    m = implem.G5Mesh()
    m.n_owned, m.n_outside, m.n_inst = t.n_owned, t.n_outside, t.n_inst
    for k, v in keep.items():
        setattr(m, k, v.ctypes.data_as(ctypes.c_void_p) if v.size else None)
    return m, keep


def _step_static(lib, prm, mesh, U, U2, dt, mode, inv, status):
    dt = np.ascontiguousarray(np.broadcast_to(np.asarray(dt, np.float64), (mesh.n_inst,)))
    rc = lib.g5_step_static(
        ctypes.byref(prm),
        ctypes.byref(mesh),
        ctypes.c_void_p(U.data_ptr()),
        ctypes.c_void_p(U2.data_ptr()),
        dt.ctypes.data_as(ctypes.c_void_p),
        implem.MODES[mode],
        ctypes.c_void_p(inv.data_ptr()),
        ctypes.c_void_p(status.data_ptr()),
        ctypes.c_void_p(torch.cuda.current_stream().cuda_stream),
    )
    assert rc == 0, rc


@pytest.mark.parametrize("mode", ["fp64", "mixed"])
def test_step_static_matches_g5_step(mode):
    lib = implem.load_library()
    mesh, t = amr_mesh(dim=2, b=8, nref=4, seed=2, periodic=False)
    p = water_air_params(t, bc=(2, 2, 3, 3, 1, 1))
    U0 = smooth_state(mesh, t, p, seed=1)
    assert (t.nbr_rel != 0).any()  # coarse/fine faces: the face-record scratch is used

    ref_impl = GodunovImplemGB300(p, t)
    A = torch.from_numpy(U0.copy()).cuda()
    ref_impl.fill_outside_quadrants(A)
    prm = implem.make_params(p)
    hmesh, _keep = _host_mesh(t)

    R0 = A.clone()
    S0 = A.clone()
    for call in range(2):  # two calls in a row
        dt = ref_impl.compute_dt_local(R0).cpu().numpy()
        R1 = torch.zeros_like(R0)
        S1 = torch.zeros_like(S0)
        inv_r = torch.zeros(t.n_inst, dtype=torch.float64, device="cuda")
        inv_s = torch.zeros(t.n_inst, dtype=torch.float64, device="cuda")
        status = torch.zeros(1, dtype=torch.int32, device="cuda")
        ref_impl.do_time_step(R0, R1, dt, mode=mode, inv_dt_out=inv_r)
        _step_static(lib, prm, hmesh, S0, S1, dt, mode, inv_s, status)
        torch.cuda.synchronize()
        n = t.n_owned
        assert torch.equal(S1[:n], R1[:n]), f"call {call}: {(S1[:n] != R1[:n]).sum().item()} values differ"
        assert torch.equal(inv_s, inv_r)
        assert status.item() == 0
        assert ref_impl.status() == 0
        ref_impl.fill_outside_quadrants(R1)
        ref_impl.fill_outside_quadrants(S1)
        R0, S0 = R1, S1


def test_step_static_rejects_oversized_and_bad_arguments():
    lib = implem.load_library()
    mesh, t = amr_mesh(dim=2, b=8, nref=2)
    p = water_air_params(t)
    prm = implem.make_params(p)
    hmesh, _keep = _host_mesh(t)
    A = torch.zeros((t.n_total, t.nv, t.ncell), dtype=torch.float64, device="cuda")
    B = torch.zeros_like(A)
    inv = torch.zeros(1, dtype=torch.float64, device="cuda")
    dt = np.ones(1)
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    vp = ctypes.c_void_p
    # same buffer as input and output
    assert lib.g5_step_static(ctypes.byref(prm), ctypes.byref(hmesh), vp(A.data_ptr()), vp(A.data_ptr()), dt.ctypes.data_as(vp), 0, vp(inv.data_ptr()), None, s) == -1
    # non-positive dt
    bad = np.zeros(1)
    assert lib.g5_step_static(ctypes.byref(prm), ctypes.byref(hmesh), vp(A.data_ptr()), vp(B.data_ptr()), bad.ctypes.data_as(vp), 0, vp(inv.data_ptr()), None, s) == -1
    # a table needing more than the fixed scratch: claim a huge block count
    big = implem.G5Mesh()
    big.n_owned = 2_000_000
    big.n_outside = 0
    big.n_inst = 1
    lv = np.zeros(big.n_owned, np.int32)
    co = np.zeros(3 * big.n_owned, np.int32)
    nb = np.zeros(9 * 4 * big.n_owned, np.int32)
    rel = np.zeros(9 * big.n_owned, np.int8)
    big.level, big.coord = lv.ctypes.data_as(vp), co.ctypes.data_as(vp)
    big.nbr, big.nbr_rel = nb.ctypes.data_as(vp), rel.ctypes.data_as(vp)
    assert lib.g5_step_static(ctypes.byref(prm), ctypes.byref(big), vp(A.data_ptr()), vp(B.data_ptr()), dt.ctypes.data_as(vp), 0, vp(inv.data_ptr()), None, s) == -1
