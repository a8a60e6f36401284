"""The five benchmark configurations of the scheme, at their full sizes and
step counts where the oracle finishes in seconds, against the CPU oracle.

* gas-water shock tube (512x32 cells, 16x16 blocks, minmod, 200 steps);
* air-helium shock-bubble (levels 4..6 of a 4x1 brick, 16x16 blocks, finest
  dx 1/1024, refined from the initial condition, 500 steps);
* air-R22 shock-bubble with THINC (beta 1.6, eps 1e-3) on the same mesh:
  one step and 500 steps, with the interface-position error;
* batched droplet-advection instances of uneven sizes (sides 64..512, a dt
  per instance): the full 256-instance batch for one step, and the first 24
  instances for 100 steps through g5_step_dev, g5_step_batched (work lists)
  and the g5_advance graph;
* 3D triple point with THINC on levels 0..3 (8^3 blocks), one step.

FP64 form: bit-exact against the oracle (so the full-run L1 error is 0, below
the 1e-10 bar).  Mixed form: volume-weighted relative L1 <= 1e-5 per
conservative variable against the oracle after the same steps.
"""
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from godunov_five_eq_gb300 import configs  # noqa: E402
from godunov_five_eq_gb300.implem import GodunovImplemGB300  # noqa: E402
from godunov_five_eq_gb300.metrics import interface_error, l1_relative  # noqa: E402
from oracle.oracle import Oracle, oracle_flag_fn  # noqa: E402

pytestmark = pytest.mark.gpu

L1_TOL_MIXED = 1e-5
L1_TOL_FP64_RUN = 1e-10
NTHREADS = os.cpu_count() or 1


def _oracle(t, p):
    return Oracle(t, p, nthreads=NTHREADS)


def _gpu_run(impl, U, nsteps, mode):
    d_U = torch.from_numpy(np.ascontiguousarray(U).copy()).cuda()
    d_U2 = torch.zeros_like(d_U)
    hist = torch.zeros(nsteps * impl.table.n_inst, dtype=torch.float64, device="cuda")
    impl.run(d_U, d_U2, nsteps, mode=mode, dt_hist=hist if mode == "fp64" else None)
    torch.cuda.synchronize()
    assert impl.status() == 0
    return d_U.cpu().numpy(), hist.cpu().numpy()


def _check_run(t, p, U, nsteps, check_interface=False):
    o = _oracle(t, p)
    ref, dts = o.run(U, nsteps)
    o.close()
    impl = GodunovImplemGB300(p, t)
    n = t.n_owned
    got, hist = _gpu_run(impl, U, nsteps, "fp64")
    assert np.array_equal(hist, dts.reshape(-1)), "dt history differs"
    diff = np.argwhere(got[:n] != ref[:n])
    assert diff.size == 0, f"FP64 after {nsteps} steps: {len(diff)} values differ, first {diff[:5]}"
    assert l1_relative(t, got, ref).max() <= L1_TOL_FP64_RUN
    mixed, _ = _gpu_run(impl, U, nsteps, "mixed")
    assert np.all(np.isfinite(mixed[:n]))
    err = l1_relative(t, mixed, ref)
    assert err.max() <= L1_TOL_MIXED, err
    if check_interface:
        ie = interface_error(t, mixed, ref)
        # the bubble (alpha_1 > 0.5): its volume, centroid and extent against
        # the FP64 oracle; shifts measured in finest cells
        assert ie is not None
        assert ie["volume_rel_diff"] <= 1e-4, ie
        assert ie["centroid_distance"] <= 0.05 * ie["finest_dx"], ie
        assert ie["extent_max_shift"] <= 1.0 * ie["finest_dx"], ie
    impl.close()


def _check_one_step(t, p, U):
    o = _oracle(t, p)
    U = np.ascontiguousarray(U).copy()
    o.fill_outside(U)
    dt = o.dt(U)
    ref = o.step(U, dt)
    o.fill_outside(ref)
    inv_ref = o.inv_dt(ref)
    o.close()
    impl = GodunovImplemGB300(p, t)
    d_U = torch.from_numpy(U).cuda()
    n = t.n_owned
    for mode in ("fp64", "mixed"):
        d_U2 = torch.zeros_like(d_U)
        inv = torch.zeros(t.n_inst, dtype=torch.float64, device="cuda")
        impl.do_time_step(d_U, d_U2, dt, mode=mode, inv_dt_out=inv)
        torch.cuda.synchronize()
        assert impl.status() == 0
        got = d_U2.cpu().numpy()
        if mode == "fp64":
            diff = np.argwhere(got[:n] != ref[:n])
            assert diff.size == 0, f"{len(diff)} values differ, first {diff[:5]}"
            assert np.array_equal(inv.cpu().numpy(), inv_ref)
        else:
            err = l1_relative(t, got, ref)
            assert err.max() <= L1_TOL_MIXED, err
    impl.close()


def test_gas_water_shock_tube_200_steps():
    """512x32 cells, water (stiffened gas) | air, minmod, HLLC, 200 steps."""
    mesh, t, p, U = configs.gas_water_shock_tube()
    assert t.n_owned * t.ncell == 512 * 32
    _check_run(t, p, U, 200)


def test_shock_bubble_air_helium_500_steps():
    """Levels 4..6, 16x16 blocks, finest dx 1/1024, 500 steps."""
    mesh, t, p, U = configs.shock_bubble("helium", thinc=False, flag_fn=oracle_flag_fn())
    assert t.level_dx[6] == pytest.approx(1.0 / 1024)
    _check_run(t, p, U, 500)


def test_shock_bubble_air_r22_thinc_one_step():
    mesh, t, p, U = configs.shock_bubble("r22", thinc=True, flag_fn=oracle_flag_fn())
    assert p.thinc == 1 and p.thinc_beta == 1.6
    _check_one_step(t, p, U)


def test_shock_bubble_air_r22_thinc_500_steps():
    mesh, t, p, U = configs.shock_bubble("r22", thinc=True, flag_fn=oracle_flag_fn())
    _check_run(t, p, U, 500, check_interface=True)


def test_triple_point_3d_levels_0_3_one_step():
    """The 3D triple point at its benchmark size (13k blocks of 8^3, 6.9 M cells)."""
    mesh, t, p, U = configs.triple_point_3d(flag_fn=oracle_flag_fn())
    assert t.level[: t.n_owned].max() == 3
    _check_one_step(t, p, U)


def test_droplet_batch_256_instances_one_step():
    """The full batch: 256 periodic instances of sides 64..512, a dt each."""
    _, t, p, U, specs = configs.droplet_instances()
    assert t.n_inst == 256 and len({s[0] for s in specs}) == 4
    _check_one_step(t, p, np.ascontiguousarray(U))


def _full_U(t, U):
    A = np.zeros((t.n_total, t.nv, t.ncell))
    A[: t.n_owned] = U[: t.n_owned]
    return A


def test_droplet_batch_100_steps_dev_batched_and_graph():
    """24 uneven instances, 100 steps, against the oracle's loop (dt per
    instance): (1) g5_step_dev with the device dt, (2) g5_step_batched over
    two work lists that together cover every instance, (3) the g5_advance
    graph loop (g5_run)."""
    _, t, p, U, specs = configs.droplet_instances(n_inst=24)
    assert len({s[0] for s in specs}) >= 3
    U = _full_U(t, U)
    nsteps = 100
    o = _oracle(t, p)
    ref, dts = o.run(U, nsteps)
    assert len(np.unique(dts[0])) > 1  # the instances do step with their own dt
    n = t.n_owned
    impl = GodunovImplemGB300(p, t)
    lists = [list(range(0, t.n_inst, 2)), list(range(1, t.n_inst, 2))]
    for path in ("dev", "batched"):
        for mode in ("fp64", "mixed"):
            A = torch.from_numpy(U.copy()).cuda()
            B = torch.zeros_like(A)
            for _ in range(nsteps):
                impl.fill_outside_quadrants(A)
                dt = impl.compute_dt_local(A)
                if path == "dev":
                    impl.do_time_step_dev(A, B, dt, mode=mode)
                else:
                    for lst in lists:
                        impl.do_time_step_batched(A, B, dt, lst, mode=mode)
                A, B = B, A
            impl.fill_outside_quadrants(A)
            torch.cuda.synchronize()
            assert impl.status() == 0
            got = A.cpu().numpy()
            if mode == "fp64":
                assert np.array_equal(got[:n], ref[:n]), f"{path}: {(got[:n] != ref[:n]).sum()} values differ"
            else:
                err = l1_relative(t, got, ref)
                assert err.max() <= L1_TOL_MIXED, (path, err)
    got, hist = _gpu_run(impl, U, nsteps, "fp64")
    assert np.array_equal(hist, dts.reshape(-1))
    assert np.array_equal(got[:n], ref[:n])
    mixed, _ = _gpu_run(impl, U, nsteps, "mixed")
    assert l1_relative(t, mixed, ref).max() <= L1_TOL_MIXED
    o.close()
    impl.close()
