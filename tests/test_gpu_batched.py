"""g5_step_batched: one step of a work list of instances.

The listed instances' owned blocks must come out bit-identical to a full
g5_step of the whole batch (both precision modes, with and without
coarse/fine records); the other instances' blocks of U2 and their CFL
accumulators must stay untouched.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from godunov_five_eq_gb300 import configs  # noqa: E402
from godunov_five_eq_gb300.implem import G5Error, GodunovImplemGB300  # noqa: E402
from godunov_five_eq_gb300.mesh import concat_tables  # noqa: E402
from tests.helpers import amr_mesh, smooth_state, water_air_params  # noqa: E402

pytestmark = pytest.mark.gpu

SENTINEL = -3.25


def _droplets():
    meshes, t, p, U, specs = configs.droplet_instances(n_inst=5, sides=(64, 128))
    return t, p, U


def _amr_pair():
    ts, Us = [], []
    for seed in (0, 4):
        mesh, t = amr_mesh(dim=2, b=8, nref=3, seed=seed)
        p = water_air_params(t)
        ts.append(t)
        Us.append(smooth_state(mesh, t, p, seed=seed))
    t = concat_tables(ts)
    U = np.concatenate([Us[0][: ts[0].n_owned], Us[1][: ts[1].n_owned], Us[0][ts[0].n_owned :], Us[1][ts[1].n_owned :]])
    return t, water_air_params(t), U


@pytest.mark.parametrize("case", ["droplets", "amr_pair"])
@pytest.mark.parametrize("mode", ["fp64", "mixed"])
def test_batched_matches_full_step(case, mode):
    t, p, U = _droplets() if case == "droplets" else _amr_pair()
    impl = GodunovImplemGB300(p, t)
    A = torch.from_numpy(np.ascontiguousarray(U)).cuda()
    impl.fill_outside_quadrants(A)
    dt = impl.compute_dt_local(A)
    full = torch.zeros_like(A)
    inv_full = torch.zeros(t.n_inst, dtype=torch.float64, device="cuda")
    impl.do_time_step_dev(A, full, dt, mode=mode, inv_dt_out=inv_full)
    listed = [t.n_inst - 1] if case == "amr_pair" else [0, 3, 4]
    part = torch.full_like(A, SENTINEL)
    inv_part = torch.zeros(t.n_inst, dtype=torch.float64, device="cuda")
    impl.do_time_step_batched(A, part, dt, listed, mode=mode, inv_dt_out=inv_part)
    torch.cuda.synchronize()
    assert impl.status() == 0
    n = t.n_owned
    inst = np.asarray(t.inst[:n])
    sel = np.isin(inst, listed)
    F, P = full.cpu().numpy(), part.cpu().numpy()
    assert sel.any() and (~sel).any()
    assert np.array_equal(P[:n][sel], F[:n][sel])
    assert np.all(P[:n][~sel] == SENTINEL)
    assert np.all(P[n:] == SENTINEL)
    ip, ifull = inv_part.cpu().numpy(), inv_full.cpu().numpy()
    for i in range(t.n_inst):
        assert ip[i] == (ifull[i] if i in listed else 0.0)


def test_batched_rejects_bad_instance():
    t, p, U = _droplets()
    impl = GodunovImplemGB300(p, t)
    A = torch.from_numpy(np.ascontiguousarray(U)).cuda()
    dt = impl.compute_dt_local(A)
    with pytest.raises(G5Error):
        impl.do_time_step_batched(A, torch.zeros_like(A), dt, [t.n_inst])
    # an empty list is a no-op
    B = torch.full_like(A, SENTINEL)
    impl.do_time_step_batched(A, B, dt, [])
    torch.cuda.synchronize()
    assert torch.all(B == SENTINEL)


def test_tail_reflux_counters_over_many_steps():
    """The FP32-bulk 2D step finishes the coarse/fine records in its tail by
    arrival counters and ticket claims that reset themselves: 30 graph-replayed
    steps of a two-instance AMR batch give the same bits as the separate
    reflux pass, and the counters end where they started (a second run
    repeats the first)."""
    t, p, U = _amr_pair()
    assert (t.nbr_rel != 0).any()
    impl = GodunovImplemGB300(p, t)
    n = t.n_owned

    def run(layout):
        impl.set_shape("mixed", reflux_layout=layout)
        A = torch.from_numpy(np.ascontiguousarray(U).copy()).cuda()
        B = torch.zeros_like(A)
        impl.run(A, B, 30, "mixed")
        torch.cuda.synchronize()
        assert impl.status() == 0
        return A.cpu().numpy()[:n]

    tail = run(2)
    assert np.array_equal(run(0), tail)
    assert np.array_equal(run(2), tail)
    impl.close()
