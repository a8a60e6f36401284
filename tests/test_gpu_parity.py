"""GPU path (through the C ABI) against the CPU oracle.

FP64 mode: bit-exact (the kernels are compiled without multiply-add
contraction and evaluate every expression in the reference's order).
Mixed mode (FP32 bulk): volume-weighted relative L1 error per conservative
variable <= 1e-5 against the FP64 oracle after the same number of steps.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from godunov_five_eq_gb300 import configs  # noqa: E402
from godunov_five_eq_gb300.implem import G5Error, GodunovImplemGB300  # noqa: E402
from godunov_five_eq_gb300.mesh import BlockMesh  # noqa: E402
from oracle.oracle import Oracle, oracle_flag_fn  # noqa: E402
from tests.helpers import amr_mesh, smooth_state, water_air_params  # noqa: E402

pytestmark = pytest.mark.gpu

L1_TOL_MIXED = 1e-5


def l1_rel(t, A, B):
    """Volume-weighted relative L1 error per conservative variable.  Momentum
    components are normalised by the momentum magnitude |rho u| (a component
    that is zero in the reference, e.g. rho v before the shock meets the
    bubble, would otherwise divide by round-off)."""
    from godunov_five_eq_gb300.metrics import l1_relative

    return l1_relative(t, A, B)


def gpu_one_step(t, p, U, dt, mode="fp64"):
    impl = GodunovImplemGB300(p, t)
    d_U = torch.from_numpy(U).cuda()
    d_U2 = torch.zeros_like(d_U)
    inv = torch.zeros(t.n_inst, dtype=torch.float64, device="cuda")
    impl.do_time_step(d_U, d_U2, dt, mode=mode, inv_dt_out=inv)
    torch.cuda.synchronize()
    assert impl.status() == 0
    return d_U2.cpu().numpy(), inv.cpu().numpy(), impl


def cases():
    out = []
    # 1) gas-water shock tube (ZERO_GRADIENT x, periodic y), 16^2 blocks
    mesh, t, p, U = configs.gas_water_shock_tube()
    out.append(("shock_tube_16", t, p, U))
    # 2) periodic 3-level AMR, 8^2 blocks, smooth interface
    mesh, t = amr_mesh(dim=2, b=8, nref=3, seed=0)
    p = water_air_params(t)
    out.append(("amr_periodic_8", t, p, smooth_state(mesh, t, p)))
    # 3) walls and zero-gradient with AMR at the boundaries (outside blocks at several levels)
    mesh, t = amr_mesh(dim=2, b=8, nref=4, seed=2, periodic=False)
    p = water_air_params(t, bc=(2, 2, 3, 3, 1, 1))
    out.append(("amr_walls_8", t, p, smooth_state(mesh, t, p, seed=1)))
    # 4) same with THINC and MC slopes
    p2 = water_air_params(t, bc=(2, 2, 3, 3, 1, 1), thinc=1, slope_type=2.0)
    out.append(("amr_walls_thinc_8", t, p2, smooth_state(mesh, t, p2, seed=1)))
    # 5) RK1 (no Hancock predictor)
    p3 = water_air_params(t, bc=(2, 2, 3, 3, 1, 1), integrator=1)
    out.append(("amr_walls_rk1_8", t, p3, smooth_state(mesh, t, p3, seed=1)))
    # 6) shock-bubble (air-helium) on 16^2 blocks, 3 levels from the refine flags
    mesh, t, p, U = configs.shock_bubble(level_min=2, level_max=4, flag_fn=oracle_flag_fn())
    out.append(("shock_bubble_16", t, p, U))
    return out


CASES = cases()


@pytest.mark.parametrize("name,t,p,U", CASES, ids=[c[0] for c in CASES])
def test_fp64_one_step_bit_exact(name, t, p, U):
    o = Oracle(t, p)
    U = U.copy()
    o.fill_outside(U)
    dt = o.dt(U)
    ref = o.step(U, dt)
    got, inv, _ = gpu_one_step(t, p, U, dt)
    n = t.n_owned
    diff = np.argwhere(got[:n] != ref[:n])
    assert diff.size == 0, f"{len(diff)} values differ, first {diff[:5]}"
    # fused CFL reduction of the new state == ComputeDtFiveEqFunctor on U2
    o.fill_outside(ref)
    assert np.array_equal(inv, o.inv_dt(ref))


@pytest.mark.parametrize("name,t,p,U", CASES[:3], ids=[c[0] for c in CASES[:3]])
def test_inv_dt_and_fill_outside_exact(name, t, p, U):
    o = Oracle(t, p)
    Uo = U.copy()
    o.fill_outside(Uo)
    impl = GodunovImplemGB300(p, t)
    d = torch.from_numpy(U.copy()).cuda()
    impl.fill_outside_quadrants(d)
    inv = impl.compute_inv_dt(d)
    torch.cuda.synchronize()
    assert np.array_equal(d.cpu().numpy(), Uo)
    assert np.array_equal(inv.cpu().numpy(), o.inv_dt(Uo))


@pytest.mark.parametrize("name,t,p,U", [CASES[1], CASES[2], CASES[5]], ids=["amr_periodic_8", "amr_walls_8", "shock_bubble_16"])
def test_fp64_run_bit_exact(name, t, p, U):
    nsteps = 7
    o = Oracle(t, p)
    ref, dts = o.run(U, nsteps)
    impl = GodunovImplemGB300(p, t)
    d_U = torch.from_numpy(U.copy()).cuda()
    d_U2 = torch.zeros_like(d_U)
    hist = torch.zeros(nsteps * t.n_inst, dtype=torch.float64, device="cuda")
    impl.run(d_U, d_U2, nsteps, mode="fp64", dt_hist=hist)
    torch.cuda.synchronize()
    assert np.array_equal(hist.cpu().numpy(), dts.reshape(-1))
    assert np.array_equal(d_U.cpu().numpy()[: t.n_owned], ref[: t.n_owned])
    # graph-replayed loop (no dt history) gives the same state
    d_U = torch.from_numpy(U.copy()).cuda()
    impl.run(d_U, d_U2, nsteps, mode="fp64")
    torch.cuda.synchronize()
    assert np.array_equal(d_U.cpu().numpy()[: t.n_owned], ref[: t.n_owned])
    assert impl.status() == 0


@pytest.mark.parametrize("name,t,p,U", CASES, ids=[c[0] for c in CASES])
def test_mixed_l1_error(name, t, p, U):
    nsteps = 10
    o = Oracle(t, p)
    ref, _ = o.run(U, nsteps)
    impl = GodunovImplemGB300(p, t)
    d_U = torch.from_numpy(U.copy()).cuda()
    d_U2 = torch.zeros_like(d_U)
    impl.run(d_U, d_U2, nsteps, mode="mixed")
    torch.cuda.synchronize()
    got = d_U.cpu().numpy()
    assert np.all(np.isfinite(got[: t.n_owned]))
    err = l1_rel(t, got, ref)
    assert err.max() <= L1_TOL_MIXED, err


def test_refine_flags_exact():
    for ind in (0, 1, 2):
        mesh, t = amr_mesh(dim=2, b=8, nref=4, seed=2, periodic=False)
        p = water_air_params(t, bc=(2, 2, 3, 3, 1, 1))
        U = smooth_state(mesh, t, p, seed=1)
        o = Oracle(t, p)
        o.fill_outside(U)
        ref = o.refine_flags(U, ind, 0.1, 0.0125, 0.02, 1, 3)
        impl = GodunovImplemGB300(p, t)
        got = impl.refine_flags(torch.from_numpy(U).cuda(), ind, 0.1, 0.0125, 0.02, 1, 3).cpu().numpy()
        assert np.array_equal(got, ref), ind


@pytest.mark.parametrize("mode", ["fp64", "mixed"])
@pytest.mark.parametrize("var", [1, 2, 7])
def test_nonphysical_input_raises_status_not_fault(mode, var):
    """A NaN planted on the host in one cell (energy, momentum or a partial
    density) raises the status word in both precision forms, and every value
    the FP64 oracle turns non-finite is non-finite on the GPU too: the mixed
    path's double -> float conversion must carry the NaN into the neighbours'
    fluxes, not a finite stand-in."""
    mesh, t = amr_mesh(dim=2, b=8, nref=2)
    p = water_air_params(t)
    U = smooth_state(mesh, t, p)
    U[0, var, 5 * 8 + 5] = np.nan
    o = Oracle(t, p)
    o.fill_outside(U)
    ref = o.step(U, 1e-7)
    impl = GodunovImplemGB300(p, t)
    d_U = torch.from_numpy(U).cuda()
    d_U2 = torch.zeros_like(d_U)
    impl.do_time_step(d_U, d_U2, 1e-7, mode=mode)
    assert impl.status() & 1
    assert impl.status() == 0  # cleared by the read
    n = t.n_owned
    got = d_U2.cpu().numpy()[:n]
    bad_ref = ~np.isfinite(ref[:n])
    assert bad_ref.any()
    assert np.all(~np.isfinite(got[bad_ref]))
    if mode == "fp64":
        assert np.array_equal(~np.isfinite(got), bad_ref)


def test_bad_mesh_rejected():
    mesh, t = amr_mesh(dim=2, b=8, nref=2)
    p = water_air_params(t)
    t.nbr[0, 0, 0] = t.n_total + 5
    with pytest.raises(G5Error):
        GodunovImplemGB300(p, t)


@pytest.mark.parametrize("thinc", [0, 1])
def test_rk2_ssp_run_fp64_exact_and_mixed(thinc):
    """RK2_SSP solver loop (two stages + 0.5 U + 0.5 U2) against the oracle's loop."""
    mesh, t = amr_mesh(dim=2, b=8, nref=4, seed=2, periodic=False)
    p = water_air_params(t, bc=(2, 2, 3, 3, 1, 1), thinc=thinc, integrator=2)
    U = smooth_state(mesh, t, p, seed=1)
    nsteps = 5
    o = Oracle(t, p)
    ref, dts = o.run(U, nsteps)
    impl = GodunovImplemGB300(p, t)
    hist = torch.zeros(nsteps, dtype=torch.float64, device="cuda")
    d_U = torch.from_numpy(U.copy()).cuda()
    d_U2 = torch.zeros_like(d_U)
    impl.run(d_U, d_U2, nsteps, mode="fp64", dt_hist=hist)
    torch.cuda.synchronize()
    assert np.array_equal(hist.cpu().numpy(), dts.reshape(-1))
    assert np.array_equal(d_U.cpu().numpy()[: t.n_owned], ref[: t.n_owned])
    d_U = torch.from_numpy(U.copy()).cuda()
    impl.run(d_U, d_U2, nsteps, mode="mixed")
    torch.cuda.synchronize()
    from godunov_five_eq_gb300.metrics import l1_relative

    assert l1_relative(t, d_U.cpu().numpy(), ref).max() <= L1_TOL_MIXED
    assert impl.status() == 0


@pytest.mark.parametrize("dim", [2, 3])
def test_miller_puckett_source_term(dim):
    """MILLER_PUCKETT volume-fraction source term (get_source_term_factor,
    ReadFluxesAndConservativeUpdateFunctor.h:412-443): FP64 bit-exact, mixed L1."""
    b = 8
    if dim == 2:
        mesh, t = amr_mesh(dim=2, b=b, nref=4, seed=2, periodic=False)
        bc = (2, 2, 3, 3, 1, 1)
    else:
        mesh, t = amr_mesh(dim=3, b=b, nref=2, seed=3, periodic=False, nbrick=(2, 1, 1), lmin=1, lmax=2)
        bc = (2, 2, 3, 3, 2, 3)
    p = water_air_params(t, dim=dim, b=b, bc=bc, source_term=1)
    U = smooth_state(mesh, t, p, seed=1)
    nsteps = 3
    o = Oracle(t, p)
    ref, _ = o.run(U, nsteps)
    impl = GodunovImplemGB300(p, t)
    from godunov_five_eq_gb300.metrics import l1_relative

    for mode in ("fp64", "mixed"):
        d_U = torch.from_numpy(U.copy()).cuda()
        d_U2 = torch.zeros_like(d_U)
        impl.run(d_U, d_U2, nsteps, mode=mode)
        torch.cuda.synchronize()
        got = d_U.cpu().numpy()
        if mode == "fp64":
            assert np.array_equal(got[: t.n_owned], ref[: t.n_owned])
        else:
            assert l1_relative(t, got, ref).max() <= L1_TOL_MIXED
    assert impl.status() == 0
