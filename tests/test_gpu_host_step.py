"""g5_step_host (host U/U2, chunked copies overlapped with the step) against
g5_step on device buffers and against the oracle.

The pipelined path steps the blocks in a different order (chunk by chunk as
their neighbours arrive) and refluxes coarse/fine records per chunk; every
block's arithmetic is unchanged, so the results are bit-identical to g5_step
in both precision modes and, in FP64, to the oracle.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from godunov_five_eq_gb300 import configs  # noqa: E402
from godunov_five_eq_gb300.implem import G5Error, GodunovImplemGB300  # noqa: E402
from oracle.oracle import Oracle, oracle_flag_fn  # noqa: E402
from tests.helpers import amr_mesh, smooth_state, water_air_params  # noqa: E402

pytestmark = pytest.mark.gpu


def _cases():
    out = []
    mesh, t, p, U = configs.shock_bubble(level_min=2, level_max=4, bsize=8, flag_fn=oracle_flag_fn())
    out.append(("shock_bubble_8", t, p, U))
    mesh, t, p, U = configs.shock_bubble(level_min=3, level_max=5, bsize=16, flag_fn=oracle_flag_fn(), thinc=True)
    out.append(("shock_bubble_16_thinc", t, p, U))
    mesh, t = amr_mesh(dim=3, b=8, nref=2, seed=3, periodic=False, nbrick=(2, 2, 2))
    p = water_air_params(t, dim=3, b=8, bc=(2, 2, 3, 3, 2, 2))
    out.append(("amr3d_walls", t, p, smooth_state(mesh, t, p, seed=3)))
    return out


CASES = _cases()


@pytest.mark.parametrize("name,t,p,U", CASES, ids=[c[0] for c in CASES])
@pytest.mark.parametrize("mode", ["fp64", "mixed"])
@pytest.mark.parametrize("pinned", [True, False], ids=["pinned", "pageable"])
def test_step_host_matches_device_step(name, t, p, U, mode, pinned):
    o = Oracle(t, p)
    o.fill_outside(U)
    dt = o.dt(U)
    impl = GodunovImplemGB300(p, t)
    d_U = torch.from_numpy(U).cuda()
    d_U2 = torch.zeros_like(d_U)
    inv_d = torch.zeros(t.n_inst, dtype=torch.float64, device="cuda")
    impl.do_time_step(d_U, d_U2, dt, mode=mode, inv_dt_out=inv_d)
    hU = torch.from_numpy(U.copy())
    hO = torch.full_like(hU, -7.0)
    if pinned:  # graph replay, U2 written straight into host memory
        hU, hO = hU.pin_memory(), hO.pin_memory()
    inv_h = torch.zeros(t.n_inst, dtype=torch.float64)
    for _ in range(2):  # second call replays the cached graph / reuses the staging arrays
        impl.do_time_step_host(hU, hO, dt, mode=mode, inv_dt_out=inv_h)
        torch.cuda.synchronize()
    torch.cuda.synchronize()
    assert impl.status() == 0
    n = t.n_owned
    ref = d_U2.cpu().numpy()
    assert np.array_equal(hO.numpy()[:n], ref[:n])
    assert np.all(hO.numpy()[n:] == -7.0)  # outside blocks of U2 are not written
    assert np.array_equal(inv_h.numpy(), inv_d.cpu().numpy())
    if mode == "fp64":
        assert np.array_equal(hO.numpy()[:n], o.step(U, dt)[:n])
    if name == "shock_bubble_8":
        assert impl.last_launch_count() > 2  # several chunks


def test_step_host_rejects_device_tensors():
    mesh, t, p, U = configs.gas_water_shock_tube(bsize=8, nx_blocks=8, ny_blocks=2)
    impl = GodunovImplemGB300(p, t)
    d = torch.from_numpy(U).cuda()
    with pytest.raises(ValueError):
        impl.do_time_step_host(d, d, 1e-6)
    h = torch.from_numpy(U.copy())
    with pytest.raises(G5Error):
        impl.do_time_step_host(h, h.clone(), -1.0)
