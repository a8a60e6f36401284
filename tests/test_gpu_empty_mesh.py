"""A context whose mesh has no blocks (a rank that owns none of the forest's
leaves): every call succeeds and launches nothing, and the context steps a
real mesh afterwards exactly as a fresh one does."""
import ctypes

import numpy as np
import pytest

from godunov_five_eq_gb300 import implem
from godunov_five_eq_gb300.mesh import BlockTable
from tests.helpers import amr_mesh, smooth_state, water_air_params


def _empty_table(t):
    return BlockTable(
        dim=t.dim,
        bsize=t.bsize,
        n_owned=0,
        n_outside=0,
        level=np.zeros(0, np.int32),
        coord=np.zeros((0, 3), np.int32),
        nbr=np.zeros((0, t.nbr.shape[1], t.nbr.shape[2]), np.int32),
        nbr_rel=np.zeros((0, t.nbr_rel.shape[1]), np.int8),
        out_src=np.zeros(0, np.int32),
        out_normal=np.zeros((0, 3), np.int8),
        out_border=np.zeros((0, 6), np.int8),
        inst=np.zeros(0, np.int32),
        level_dx=t.level_dx,
    )


def test_empty_table_accepted_on_cpu_side():
    # the table builder and the argument checks need no GPU: an empty table
    # is a valid BlockTable with zero-length arrays
    mesh, t = amr_mesh(dim=2, b=8, nref=1)
    e = _empty_table(t)
    assert e.n_owned == 0 and e.n_total == 0 and e.n_inst == 1


@pytest.mark.gpu
@pytest.mark.parametrize("dim", [2, 3])
def test_empty_mesh_calls_launch_nothing(dim):
    torch = pytest.importorskip("torch")
    from oracle import oracle as orc

    mesh, t = amr_mesh(dim=dim, b=8, nref=2, seed=dim)
    p = water_air_params(t, dim=dim, b=8)
    impl = implem.GodunovImplemGB300(p, _empty_table(t))
    dummy = torch.zeros(1, dtype=torch.float64, device="cuda")
    dummy2 = torch.zeros(1, dtype=torch.float64, device="cuda")
    for mode in ("fp64", "mixed"):
        impl.do_time_step(dummy, dummy2, 1e-6, mode=mode)
        assert impl.last_launch_count() == 0
    inv = impl.compute_inv_dt(dummy)
    impl.fill_outside_quadrants(dummy)
    torch.cuda.synchronize()
    assert float(inv[0]) == 0.0
    assert impl.status() == 0
    # the same context then steps a real mesh bit for bit like the oracle
    U = smooth_state(mesh, t, p, seed=dim)
    impl.resize_auxiliary_data(t)
    A = torch.from_numpy(U).cuda()
    B = torch.zeros_like(A)
    o = orc.Oracle(t, p)
    o.fill_outside(U)
    impl.fill_outside_quadrants(A)
    dt = o.dt(U)
    impl.do_time_step(A, B, dt, mode="fp64")
    torch.cuda.synchronize()
    assert impl.status() == 0
    ref = o.step(U, dt)
    assert np.array_equal(B.cpu().numpy()[: t.n_owned], ref[: t.n_owned])
    impl.close()
