"""g5_step_static, the allocation-free step, against g5_step.

g5_step_static serves callers that must not allocate device memory while
they advance the solution (a solver whose device memory belongs to its
framework's pool allocator, or a plugin whose host process accounts for every
device allocation).  It runs the same kernels as g5_step with all scratch in
a fixed file-scope device array, so its results must equal g5_step's bit for
bit, in FP64 and in mixed mode, on two consecutive steps (the second call
reuses the array the first one filled), on 2D meshes of 8^2 and 16^2 blocks,
a 3D mesh of 8^3 blocks and two batched instances with a dt each, with and
without a caller status word.  The meshes have coarse/fine faces, so the
face-record scratch is exercised too.  A corrupted block table and a stream in
capture mode are refused.

This file is collected last so that a run stopping at the first failure has
already run every other test; it also passes alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from godunov_five_eq_gb300 import implem  # noqa: E402
from godunov_five_eq_gb300.implem import GodunovImplemGB300  # noqa: E402
from godunov_five_eq_gb300.mesh import concat_tables  # noqa: E402
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
        ctypes.c_void_p(status.data_ptr()) if status is not None else None,
        ctypes.c_void_p(torch.cuda.current_stream().cuda_stream),
    )
    assert rc == 0, rc


def _case(name):
    """Meshes with coarse/fine faces (the face-record scratch is used): 2D 8^2
    and 16^2 blocks with walls, 3D 8^3 blocks, and two 2D instances batched in
    one table with a dt each."""
    if name == "2d_b8_walls":
        mesh, t = amr_mesh(dim=2, b=8, nref=4, seed=2, periodic=False)
        p = water_air_params(t, bc=(2, 2, 3, 3, 1, 1))
        return t, p, smooth_state(mesh, t, p, seed=1)
    if name == "2d_b16_walls":
        mesh, t = amr_mesh(dim=2, b=16, nref=3, seed=5, periodic=False)
        p = water_air_params(t, b=16, bc=(2, 2, 3, 3, 1, 1))
        return t, p, smooth_state(mesh, t, p, seed=3)
    if name == "3d_b8":
        mesh, t = amr_mesh(dim=3, b=8, nref=2, seed=3, periodic=False, nbrick=(2, 1, 1), lmin=1, lmax=2)
        p = water_air_params(t, dim=3, b=8, bc=(2, 2, 3, 3, 2, 3))
        return t, p, smooth_state(mesh, t, p, seed=2)
    ts, Us = [], []
    for seed in (0, 4):
        mesh, t = amr_mesh(dim=2, b=8, nref=3, seed=seed)
        ts.append(t)
        Us.append(smooth_state(mesh, t, water_air_params(t), seed=seed))
    t = concat_tables(ts)
    U = np.concatenate([Us[0][: ts[0].n_owned], Us[1][: ts[1].n_owned], Us[0][ts[0].n_owned :], Us[1][ts[1].n_owned :]])
    return t, water_air_params(t), U


CASES = ["2d_b8_walls", "2d_b16_walls", "3d_b8", "2d_two_instances"]


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("mode", ["fp64", "mixed"])
def test_step_static_matches_g5_step(mode, case):
    lib = implem.load_library()
    t, p, U0 = _case(case)
    assert (t.nbr_rel != 0).any()  # coarse/fine faces: the face-record scratch is used

    ref_impl = GodunovImplemGB300(p, t)
    A = torch.from_numpy(np.ascontiguousarray(U0)).cuda()
    ref_impl.fill_outside_quadrants(A)
    prm = implem.make_params(p)
    hmesh, _keep = _host_mesh(t)

    R0 = A.clone()
    S0 = A.clone()
    for call in range(2):  # two calls in a row
        dt = ref_impl.compute_dt_local(R0).cpu().numpy()
        if t.n_inst > 1:
            dt = dt * np.linspace(1.0, 0.5, t.n_inst)  # a different dt per instance
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
        # the same call with the status word left to the scratch array
        S2 = torch.zeros_like(S0)
        inv_s.zero_()
        _step_static(lib, prm, hmesh, S0, S2, dt, mode, inv_s, None)
        torch.cuda.synchronize()
        assert torch.equal(S2[:n], R1[:n])
        assert torch.equal(inv_s, inv_r)
        ref_impl.fill_outside_quadrants(R1)
        ref_impl.fill_outside_quadrants(S1)
        R0, S0 = R1, S1


def test_step_static_refuses_a_capturing_stream():
    """The host arrays are staged at call time: a stream in capture mode is
    refused (G5_ERR_UNSUPPORTED) before anything is enqueued."""
    lib = implem.load_library()
    t, p, U0 = _case("2d_b8_walls")
    prm = implem.make_params(p)
    hmesh, _keep = _host_mesh(t)
    A = torch.from_numpy(np.ascontiguousarray(U0)).cuda()
    B = torch.zeros_like(A)
    inv = torch.zeros(1, dtype=torch.float64, device="cuda")
    dt = np.full(1, 1e-7)
    x = torch.zeros(4, device="cuda")
    vp = ctypes.c_void_p
    s = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    rc = None
    with torch.cuda.graph(g, stream=s):
        x.add_(1.0)
        rc = lib.g5_step_static(
            ctypes.byref(prm), ctypes.byref(hmesh), vp(A.data_ptr()), vp(B.data_ptr()), dt.ctypes.data_as(vp), 0, vp(inv.data_ptr()), None, vp(s.cuda_stream)
        )
    assert rc == -6
    g.replay()
    torch.cuda.synchronize()
    assert torch.all(x == 1.0)


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
    # a finer slot with a needed child missing (-1): refused like g5_set_mesh refuses it
    mesh2, t2 = amr_mesh(dim=2, b=8, nref=4, seed=2, periodic=False)
    fine = np.argwhere(t2.nbr_rel == 1)
    assert fine.size
    n, sl = fine[0]
    d = (sl % 3 - 1, sl // 3 - 1)
    ch = next(c for c in range(4) if all(not ((d[e] == -1 and (c >> e) & 1 != 1) or (d[e] == 1 and (c >> e) & 1 != 0)) for e in range(2)))
    t2.nbr[n, sl, ch] = -1
    p2 = water_air_params(t2, bc=(2, 2, 3, 3, 1, 1))
    prm2 = implem.make_params(p2)
    hmesh2, _keep2 = _host_mesh(t2)
    A2 = torch.zeros((t2.n_total, t2.nv, t2.ncell), dtype=torch.float64, device="cuda")
    B2 = torch.zeros_like(A2)
    assert lib.g5_step_static(ctypes.byref(prm2), ctypes.byref(hmesh2), vp(A2.data_ptr()), vp(B2.data_ptr()), dt.ctypes.data_as(vp), 0, vp(inv.data_ptr()), None, s) == -5
    with pytest.raises(implem.G5Error):
        GodunovImplemGB300(p2, t2)
