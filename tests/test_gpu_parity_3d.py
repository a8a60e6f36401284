"""3D GPU path (8^3 blocks, through the C ABI) against the CPU oracle:
FP64 bit-exact, mixed-precision L1 <= 1e-5 (see test_gpu_parity.py)."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from godunov_five_eq_gb300 import configs  # noqa: E402
from godunov_five_eq_gb300.implem import GodunovImplemGB300  # noqa: E402
from godunov_five_eq_gb300.metrics import l1_relative  # noqa: E402
from oracle.oracle import Oracle, oracle_flag_fn  # noqa: E402
from tests.helpers import amr_mesh, smooth_state, water_air_params  # noqa: E402

pytestmark = pytest.mark.gpu


def cases3d():
    out = []
    mesh, t = amr_mesh(dim=3, b=8, nref=2, seed=0, nbrick=(2, 2, 2), lmin=1, lmax=2)
    p = water_air_params(t, dim=3, b=8)
    out.append(("amr3d_periodic", t, p, smooth_state(mesh, t, p)))
    mesh, t = amr_mesh(dim=3, b=8, nref=2, seed=3, periodic=False, nbrick=(2, 1, 1), lmin=1, lmax=2)
    p = water_air_params(t, dim=3, b=8, bc=(2, 2, 3, 3, 2, 3))
    out.append(("amr3d_walls", t, p, smooth_state(mesh, t, p, seed=2)))
    p2 = water_air_params(t, dim=3, b=8, bc=(2, 2, 3, 3, 2, 3), thinc=1, slope_type=2.0)
    out.append(("amr3d_walls_thinc", t, p2, smooth_state(mesh, t, p2, seed=2)))
    mesh, t, p, U = configs.triple_point_3d(level_min=0, level_max=1, nbrick=(7, 3, 2), scaling=1.0, flag_fn=oracle_flag_fn())
    out.append(("triple_point_small", t, p, U))
    return out


CASES = cases3d()


@pytest.mark.parametrize("name,t,p,U", CASES, ids=[c[0] for c in CASES])
def test_fp64_3d_one_step_bit_exact(name, t, p, U):
    o = Oracle(t, p)
    U = U.copy()
    o.fill_outside(U)
    dt = o.dt(U)
    ref = o.step(U, dt)
    impl = GodunovImplemGB300(p, t)
    d_U = torch.from_numpy(U).cuda()
    d_U2 = torch.zeros_like(d_U)
    inv = torch.zeros(t.n_inst, dtype=torch.float64, device="cuda")
    impl.do_time_step(d_U, d_U2, dt, mode="fp64", inv_dt_out=inv)
    torch.cuda.synchronize()
    assert impl.status() == 0
    got = d_U2.cpu().numpy()
    n = t.n_owned
    diff = np.argwhere(got[:n] != ref[:n])
    assert diff.size == 0, f"{len(diff)} values differ, first {diff[:5]}"
    o.fill_outside(ref)
    assert np.array_equal(inv.cpu().numpy(), o.inv_dt(ref))


@pytest.mark.parametrize("name,t,p,U", CASES, ids=[c[0] for c in CASES])
def test_3d_run_fp64_exact_and_mixed_l1(name, t, p, U):
    nsteps = 4
    o = Oracle(t, p)
    ref, dts = o.run(U, nsteps)
    impl = GodunovImplemGB300(p, t)
    for mode in ("fp64", "mixed"):
        d_U = torch.from_numpy(U.copy()).cuda()
        d_U2 = torch.zeros_like(d_U)
        impl.run(d_U, d_U2, nsteps, mode=mode)
        torch.cuda.synchronize()
        got = d_U.cpu().numpy()
        if mode == "fp64":
            assert np.array_equal(got[: t.n_owned], ref[: t.n_owned])
        else:
            assert np.all(np.isfinite(got[: t.n_owned]))
            err = l1_relative(t, got, ref)
            assert err.max() <= 1e-5, err
    assert impl.status() == 0


def test_refine_flags_3d_exact():
    mesh, t = amr_mesh(dim=3, b=8, nref=2, seed=3, periodic=False, nbrick=(2, 1, 1), lmin=1, lmax=2)
    p = water_air_params(t, dim=3, b=8, bc=(2, 2, 3, 3, 2, 3))
    U = smooth_state(mesh, t, p, seed=2)
    o = Oracle(t, p)
    o.fill_outside(U)
    impl = GodunovImplemGB300(p, t)
    for ind in (0, 1, 2):
        ref = o.refine_flags(U, ind, 0.1, 0.0125, 0.02, 1, 3)
        got = impl.refine_flags(torch.from_numpy(U).cuda(), ind, 0.1, 0.0125, 0.02, 1, 3).cpu().numpy()
        assert np.array_equal(got, ref), ind
