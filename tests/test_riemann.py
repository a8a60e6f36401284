"""The scheme against exact solutions (no GPU, the oracle; the GPU's FP64
form equals the oracle bit for bit, the tests in test_gpu_*.py).

* Shock tubes along x on a one-block-high strip: the oracle's MUSCL-Hancock +
  HLLC solution at t_end against the exact Riemann solution (Toro's method,
  tests/exact_riemann.py), for one gas on both sides of the contact (Sod) and
  for two ideal gases (the five-equation model's material interface), with the
  L1 error falling as the mesh is refined.
* Abgrall's test: a water slab carried through air by a uniform flow at
  uniform pressure (density ratio 1000, the stiffened-gas constant) keeps
  pressure and velocity uniform to round-off (the five-equation model's
  volume-fraction transport with its non-conservative term) under RK2_SSP,
  first-order steps and THINC; under the MUSCL-Hancock predictor at CFL 0.4
  the round-off grows after some 30 steps, a property of the method that the
  last test records.
"""
import numpy as np
import pytest

from godunov_five_eq_gb300 import configs
from godunov_five_eq_gb300.mesh import BC_PERIODIC, BC_ZERO_GRADIENT, BlockMesh
from oracle.oracle import Oracle
from tests.exact_riemann import sample, star_state


def test_exact_solver_star_states():
    # the star states of three standard one-gas problems (Toro, table 4.3)
    p, u = star_state((1.0, 0.0, 1.0, 1.4), (0.125, 0.0, 0.1, 1.4))
    assert abs(p - 0.30313) < 5e-6 and abs(u - 0.92745) < 5e-6
    p, u = star_state((1.0, 0.0, 1000.0, 1.4), (1.0, 0.0, 0.01, 1.4))
    assert abs(p - 460.894) < 5e-4 and abs(u - 19.5975) < 5e-5
    p, u = star_state((1.0, -2.0, 0.4, 1.4), (1.0, 2.0, 0.4, 1.4))
    assert abs(p - 0.00189) < 5e-6 and abs(u) < 1e-12
    # pressure and velocity are continuous across the contact, also between two gases
    left, right = (1.0, 0.0, 1.0, 1.4), (0.125, 0.0, 0.1, 5.0 / 3.0)
    p, u = star_state(left, right)
    w = sample(left, right, [0.5 + u * 0.2 - 1e-9, 0.5 + u * 0.2 + 1e-9], 0.2)
    assert np.allclose(w[1], u, rtol=1e-12) and np.allclose(w[2], p, rtol=1e-12)
    assert w[3].tolist() == [0.0, 1.0]


def _strip(ncells, bsize=16):
    """[0, 1] along x in ncells cells, one block high, periodic in y."""
    trees = ncells // bsize
    mesh = BlockMesh(2, bsize, (trees, 1), (False, True), 0, 0, scaling=1.0 / trees)
    return mesh, mesh.build()


def _shock_tube(ncells, left, right, t_end):
    mesh, t = _strip(ncells)
    p = configs.HydroParams(
        dim=2,
        bsize=t.bsize,
        gamma=(left[3], right[3]),
        pinf=(0.0, 0.0),
        cfl=0.4,
        slope_type=1.0,
        bc=(BC_ZERO_GRADIENT, BC_ZERO_GRADIENT, BC_PERIODIC, BC_PERIODIC, BC_PERIODIC, BC_PERIODIC),
        level_dx=t.level_dx,
    )
    xc = configs.cell_centers(mesh, t)
    x = xc[:, 0]
    lft = x < 0.5
    eps = 1e-8
    a0 = np.where(lft, 1.0 - eps, eps)
    rho = np.where(lft, left[0], right[0])
    U = np.zeros((t.n_total, t.nv, t.ncell))
    U[: t.n_owned] = np.moveaxis(
        configs.prim_to_cons(2, p, a0, a0 * rho, (1.0 - a0) * rho, np.where(lft, left[2], right[2]), (np.where(lft, left[1], right[1]), 0.0 * x)),
        0,
        1,
    )
    o = Oracle(t, p)
    time, steps = 0.0, 0
    while time < t_end * (1.0 - 1e-14):
        o.fill_outside(U)
        dt = min(float(o.dt(U)[0]), t_end - time)
        U = o.step(U, dt)
        time += dt
        steps += 1
        assert steps < 10000
    o.close()
    I = configs.ids(2)
    rho = U[: t.n_owned, I["ID"]]
    vel = U[: t.n_owned, I["IU"]] / rho
    return x, rho, vel, U, p, t


def _l1(x, num, exact):
    # cell average of |error| over [0, 1] (every cell has the same width)
    return float(np.mean(np.abs(num - exact)))


@pytest.mark.parametrize(
    "left,right,t_end,bound",
    [
        # Sod's problem, one gas on both sides of the contact
        ((1.0, 0.0, 1.0, 1.4), (0.125, 0.0, 0.1, 1.4), 0.2, 0.012),
        # air against a monatomic gas: the contact is a material interface
        ((1.0, 0.0, 1.0, 1.4), (0.125, 0.0, 0.1, 5.0 / 3.0), 0.2, 0.012),
        # a strong shock into the lighter gas (pressure ratio 100)
        ((1.0, 0.0, 10.0, 5.0 / 3.0), (0.125, 0.0, 0.1, 1.4), 0.08, 0.03),
    ],
)
def test_shock_tube_converges_to_exact_solution(left, right, t_end, bound):
    errs = []
    for n in (128, 256):
        x, rho, vel, U, p, t = _shock_tube(n, left, right, t_end)
        # every row of the strip holds the same solution, bit for bit
        R = rho.reshape(len(rho), 16, 16)
        assert np.array_equal(R, np.broadcast_to(R[:, :1, :], R.shape))
        ex = sample(left, right, x.ravel(), t_end)
        e_rho = _l1(x, rho.ravel(), ex[0])
        e_u = _l1(x, vel.ravel(), ex[1])
        errs.append((e_rho, e_u))
        assert np.all(np.isfinite(U[: t.n_owned]))
    # within the bound at 256 cells and falling with the cell size
    assert errs[1][0] < bound, errs
    assert errs[0][0] / errs[1][0] > 1.3, errs
    assert errs[0][1] / errs[1][1] > 1.3, errs


def _abgrall(integrator, slope_type, thinc, cfl, steps):
    """Pressure and velocity deviations (relative, max over cells) after
    `steps` steps of a water slab carried through air at uniform u and p."""
    mesh = BlockMesh(2, 16, (8, 1), (True, True), 0, 0, scaling=1.0 / 8)
    t = mesh.build()
    p = configs.HydroParams(
        dim=2,
        bsize=16,
        gamma=(4.4, 1.4),
        pinf=(6e8, 0.0),
        cfl=cfl,
        slope_type=slope_type,
        integrator=integrator,
        thinc=thinc,
        level_dx=t.level_dx,
    )
    x = configs.cell_centers(mesh, t)[:, 0]
    eps = 1e-6
    a0 = np.where((x > 0.3) & (x < 0.6), 1.0 - eps, eps)
    u0, p0 = 100.0, 1e5
    U = np.zeros((t.n_total, t.nv, t.ncell))
    U[: t.n_owned] = np.moveaxis(configs.prim_to_cons(2, p, a0, a0 * 1000.0, (1.0 - a0) * 1.0, p0, (u0 + 0.0 * x, 0.0 * x)), 0, 1)
    o = Oracle(t, p)
    U2, _ = o.run(U, steps)
    o.close()
    n = t.n_owned
    I = configs.ids(2)
    a = U2[:n, I["IA0"]]
    xi = [1.0 / (g - 1.0) for g in p.gamma]
    S = a * xi[0] + (1.0 - a) * xi[1]
    PI = a * p.gamma[0] * p.pinf[0] * xi[0] + (1.0 - a) * p.gamma[1] * p.pinf[1] * xi[1]
    rho = U2[:n, I["ID"]]
    u = U2[:n, I["IU"]] / rho
    v = U2[:n, I["IV"]] / rho
    pr = (U2[:n, I["IE"]] - 0.5 * rho * (u * u + v * v) - PI) / S
    assert not np.array_equal(a, U[:n, I["IA0"]])  # the interface moved
    assert np.max(np.abs(v)) == 0.0
    return np.max(np.abs(u - u0)) / u0, np.max(np.abs(pr - p0)) / p0


@pytest.mark.parametrize(
    "integrator,slope_type,thinc,cfl,steps",
    [
        (2, 1.0, 0, 0.4, 120),  # RK2_SSP, MUSCL
        (2, 1.0, 1, 0.4, 120),  # RK2_SSP, THINC
        (0, 0.0, 0, 0.4, 120),  # first order
        (0, 0.0, 1, 0.4, 120),  # first order, THINC
        (0, 1.0, 0, 0.4, 30),  # MUSCL-Hancock, the first 30 steps
        (0, 1.0, 0, 0.2, 120),  # MUSCL-Hancock at CFL 0.2
    ],
)
def test_abgrall_interface_keeps_pressure_and_velocity(integrator, slope_type, thinc, cfl, steps):
    # uniform to the round-off of rho e - PI (PI ~ 2.3e9 in the water, p = 1e5)
    du, dp = _abgrall(integrator, slope_type, thinc, cfl, steps)
    assert du <= 1e-13 and dp <= 1e-10, (du, dp)


def test_abgrall_hancock_predictor_amplifies_round_off():
    # A property of the method, not of this build (the oracle follows the
    # reference's functors): at this 1000:1 density contact the MUSCL-Hancock
    # predictor at CFL 0.4 lets the round-off of the first steps grow by
    # about 1.5x per step until it saturates at a few percent of the pressure;
    # without the predictor (RK2_SSP above) it stays at round-off.
    du, dp = _abgrall(0, 1.0, 0, 0.4, 60)
    assert 1e-3 < dp < 0.5 and du < 1e-2, (du, dp)


@pytest.mark.gpu
def test_gpu_shock_tube_fp64_equals_oracle_and_mixed_converges():
    """The two-gas shock tube through the C ABI: the FP64 form equals the
    oracle's run bit for bit, and the FP32-bulk form lands on the exact
    solution as closely as FP64 does (L1 error within 1 % of FP64's, and
    within 1e-5 of the FP64 state)."""
    torch = pytest.importorskip("torch")
    from godunov_five_eq_gb300.implem import GodunovImplemGB300

    left, right, t_end = (1.0, 0.0, 1.0, 1.4), (0.125, 0.0, 0.1, 5.0 / 3.0), 0.2
    x, rho_o, vel_o, U_o, p, t = _shock_tube(256, left, right, t_end)
    ex = sample(left, right, x.ravel(), t_end)
    # the same initial state, rebuilt
    lft = x < 0.5
    a0 = np.where(lft, 1.0 - 1e-8, 1e-8)
    rho0 = np.where(lft, left[0], right[0])
    U0 = np.zeros((t.n_total, t.nv, t.ncell))
    U0[: t.n_owned] = np.moveaxis(configs.prim_to_cons(2, p, a0, a0 * rho0, (1.0 - a0) * rho0, np.where(lft, left[2], right[2]), (0.0 * x, 0.0 * x)), 0, 1)
    impl = GodunovImplemGB300(p, t)
    res = {}
    for mode in ("fp64", "mixed"):
        A = torch.from_numpy(U0).cuda()
        B = torch.empty_like(A)
        time = 0.0
        while time < t_end * (1.0 - 1e-14):
            impl.fill_outside_quadrants(A)
            dt = min(float(impl.compute_dt_local(A)[0]), t_end - time)
            impl.do_time_step(A, B, dt, mode=mode)
            A, B = B, A
            time += dt
        torch.cuda.synchronize()
        assert impl.status() == 0
        res[mode] = A.cpu().numpy()
    impl.close()
    I = configs.ids(2)
    n = t.n_owned
    assert np.array_equal(res["fp64"][:n], U_o[:n])
    e64 = _l1(x, rho_o.ravel(), ex[0])
    rho_m = res["mixed"][:n, I["ID"]]
    e_m = _l1(x, rho_m.ravel(), ex[0])
    assert abs(e_m - e64) <= 0.01 * e64, (e_m, e64)
    assert np.max(np.abs(rho_m - rho_o)) <= 1e-5 * np.max(rho_o)


def _shock_tube_3d(axis, ncells, left, right, t_end, bsize=8):
    """The tube along `axis` of a 3D strip one block thick in the other two
    directions (periodic there), zero-gradient ends."""
    trees = ncells // bsize
    nbrick = [1, 1, 1]
    nbrick[axis] = trees
    periodic = [True, True, True]
    periodic[axis] = False
    mesh = BlockMesh(3, bsize, tuple(nbrick), tuple(periodic), 0, 0, scaling=1.0 / trees)
    t = mesh.build()
    bc = [BC_PERIODIC] * 6
    bc[2 * axis] = bc[2 * axis + 1] = BC_ZERO_GRADIENT
    p = configs.HydroParams(
        dim=3, bsize=bsize, gamma=(left[3], right[3]), pinf=(0.0, 0.0), cfl=0.4, slope_type=1.0, bc=tuple(bc), level_dx=t.level_dx
    )
    x = configs.cell_centers(mesh, t)[:, axis]
    lft = x < 0.5
    a0 = np.where(lft, 1.0 - 1e-8, 1e-8)
    rho = np.where(lft, left[0], right[0])
    vel = [0.0 * x, 0.0 * x, 0.0 * x]
    U = np.zeros((t.n_total, t.nv, t.ncell))
    U[: t.n_owned] = np.moveaxis(configs.prim_to_cons(3, p, a0, a0 * rho, (1.0 - a0) * rho, np.where(lft, left[2], right[2]), tuple(vel)), 0, 1)
    o = Oracle(t, p)
    time = 0.0
    while time < t_end * (1.0 - 1e-14):
        o.fill_outside(U)
        dt = min(float(o.dt(U)[0]), t_end - time)
        U = o.step(U, dt)
        time += dt
    o.close()
    # the profile along the axis: one line of cells, ordered by position
    I = configs.ids(3)
    b = bsize
    loc = np.arange(b**3)
    on_line = ((loc // (b ** ((axis + 1) % 3))) % b == 0) & ((loc // (b ** ((axis + 2) % 3))) % b == 0)
    xs = x[:, on_line].ravel()
    order = np.argsort(xs, kind="stable")
    prof = {k: U[: t.n_owned, I[k]][:, on_line].ravel()[order] for k in ("ID", "IE", "IAD0", "IAD1")}
    prof["mom"] = U[: t.n_owned, I[("IU", "IV", "IW")[axis]]][:, on_line].ravel()[order]
    return xs[order], prof


def test_3d_shock_tube_same_along_every_axis_and_near_exact():
    left, right, t_end = (1.0, 0.0, 1.0, 1.4), (0.125, 0.0, 0.1, 5.0 / 3.0), 0.2
    runs = [_shock_tube_3d(axis, 128, left, right, t_end) for axis in range(3)]
    x0, p0 = runs[0]
    for axis, (x, prof) in enumerate(runs[1:], start=1):
        assert np.array_equal(x, x0)
        for k in p0:
            if axis == 1:
                # the other directions' flux differences are exact zeros and the
                # CFL rate's first sum commutes: bit for bit
                assert np.array_equal(prof[k], p0[k]), k
            else:
                # along z the CFL rate sums (c/dx + c/dy) + (c + |w|)/dz: dt
                # differs in its last bit, the profiles at round-off
                assert np.allclose(prof[k], p0[k], rtol=0, atol=1e-13), k
    ex = sample(left, right, x0, t_end)
    assert _l1(x0, p0["ID"], ex[0]) < 0.02
    assert _l1(x0, p0["mom"] / p0["ID"], ex[1]) < 0.03
