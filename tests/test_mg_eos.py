"""Mie-Grueneisen material laws (JWL, SHOCKWAVE, SHOCKWAVE2; the decks'
mg_eos_name values besides the stiffened and ideal gases).

The laws live in the reference's external kalypsso core, so they are
restated from their published forms (parity unpinned).  CPU tests check the
oracle's restatement: the laws reduce to the ideal gas when their reference
curves vanish, the mixture sound speed equals the isentropic derivative of the
pressure, uniform states stay uniform bit for bit and mass is conserved.  GPU
tests check the FP64 path bit for bit against the oracle, and the FP32-bulk
form (FP32 laws, FP64 pressure numerator) within L1 1e-5 of it.
"""
import ctypes

import numpy as np
import pytest

from godunov_five_eq_gb300 import configs
from oracle import oracle as orc
from tests.helpers import amr_mesh

LAWS = ["jwl", "shockwave", "shockwave2"]


def mg_params(table, law, other=None, dim=2, b=8, **kw):
    k0, c0 = configs.MG_LAWS[law]
    if other == "air":
        k1, c1 = configs.EOS["STIFFENED"], (0.0,) * 8
    else:
        k1, c1 = configs.MG_LAWS[other or law]
    return configs.HydroParams(
        dim=dim,
        bsize=b,
        gamma=(3.0, 1.4),
        pinf=(0.0, 0.0),
        slope_type=kw.pop("slope_type", 1.0),
        cfl=0.4,
        bc=kw.pop("bc", (configs.BC_PERIODIC,) * 6),
        level_dx=table.level_dx,
        eos=(k0, k1),
        mg=(tuple(c0), tuple(c1)),
        **kw,
    )


def mg_state(mesh, table, params, seed=0):
    """Smooth two-material state around the laws' reference densities."""
    rng = np.random.default_rng(seed)
    xc = configs.cell_centers(mesh, table)
    x, y = xc[:, 0], xc[:, 1]
    z = xc[:, 2] if table.dim == 3 else 0.0 * x
    k = rng.uniform(0.5, 1.5, size=3)
    r = np.sqrt((x - 0.8) ** 2 + (y - 0.9) ** 2 + ((z - 0.7) ** 2 if table.dim == 3 else 0.0))
    a0 = 1e-6 + (1 - 2e-6) * 0.5 * (1 - np.tanh((r - 0.4) / 0.05))
    rho0 = [params.mg[kk][0] if params.eos[kk] else 1.2 for kk in range(2)]
    ar0 = a0 * rho0[0] * (1.1 + 0.05 * np.sin(2 * np.pi * k[0] * y))
    ar1 = (1 - a0) * rho0[1] * (1.05 + 0.05 * np.cos(2 * np.pi * x))
    p = 5e9 * (1 + 0.2 * np.sin(2 * np.pi * (x + y)))
    vel = [100 * np.cos(2 * np.pi * y), -50 * np.sin(2 * np.pi * x)]
    if table.dim == 3:
        vel.append(30 * np.cos(2 * np.pi * z))
    U = np.zeros((table.n_total, table.nv, table.ncell))
    U[: table.n_owned] = np.moveaxis(configs.prim_to_cons(table.dim, params, a0, ar0, ar1, p, tuple(vel)), 0, 1)
    return U


# ------------------------------------------------------------------- oracle
@pytest.mark.parametrize("law", ["jwl", "shockwave2"])
def test_oracle_law_reduces_to_ideal_gas(law):
    """JWL with A1 = A2 = 0 and SHOCKWAVE2 with c0 = p0 = 0, alpha = 0 are the
    ideal gas gamma = Gamma0 + 1: a shock tube run through the general mixture
    rules matches the stiffened-gas path to round-off."""
    mesh, t, p_sg, U = configs.gas_water_shock_tube(nx_blocks=8)
    g = 0.4
    p_sg.gamma, p_sg.pinf = (1.0 + g, 1.0 + g), (0.0, 0.0)
    if law == "jwl":
        c = (1.0, g, 0.0, 0.0, 4.0, 1.0, 0.0, 0.0)
    else:
        c = (1.0, g, 0.0, 1.3, 0.0, 0.0, 0.0, 0.0)
    kind = configs.EOS[law.upper()]
    p_mg = configs.HydroParams(**{**p_sg.__dict__, "eos": (kind, kind), "mg": (c, c)})
    U = np.zeros_like(U)
    xc = configs.cell_centers(mesh, t)
    left = xc[:, 0] < 0.5
    a0 = np.where(left, 1 - 1e-6, 1e-6)
    st = configs.prim_to_cons(2, p_sg, a0, a0 * 3.0, (1 - a0) * 1.0, np.where(left, 10.0, 1.0), (0 * a0, 0 * a0))
    U[: t.n_owned] = np.moveaxis(st, 0, 1)
    ref, dts = orc.Oracle(t, p_sg).run(U, 20)
    got, dtg = orc.Oracle(t, p_mg).run(U, 20)
    n = t.n_owned
    assert np.allclose(dtg, dts, rtol=1e-12, atol=0)
    for v in range(t.nv):
        scale = np.abs(ref[:n, v]).max() + 1e-30
        assert np.abs(got[:n, v] - ref[:n, v]).max() <= 1e-11 * scale, v


@pytest.mark.parametrize("law", LAWS)
def test_oracle_sound_speed_is_isentropic_derivative(law):
    """c^2 = dp/drho along de = p/rho^2 drho (one material), from the oracle's
    pressure, against its sound speed."""
    mesh, t = amr_mesh(dim=2, b=8, nref=1)
    prm = orc.make_params(mg_params(t, law))
    L = orc.lib()
    rho0 = configs.MG_LAWS[law][1][0]
    for comp in (0.9, 1.0, 1.2, 1.6):
        rho = comp * rho0
        p = 3e9
        # e from p by the mixture rules (one material: a0 = 1)
        S_PI = configs.mixture_S_PI(mg_params(t, law), np.array(1.0), np.array(rho), np.array(0.0))
        e = float((p * S_PI[0] + S_PI[1]) / rho)
        c = L.g5o_mixture_sound_speed(ctypes.byref(prm), rho, p, 1.0, rho, 0.0)
        h = rho * 1e-6
        pp = L.g5o_mixture_pressure(ctypes.byref(prm), rho + h, e + p / rho**2 * h, 1.0, rho + h, 0.0)
        pm = L.g5o_mixture_pressure(ctypes.byref(prm), rho - h, e - p / rho**2 * h, 1.0, rho - h, 0.0)
        assert L.g5o_mixture_pressure(ctypes.byref(prm), rho, e, 1.0, rho, 0.0) == pytest.approx(p, rel=1e-12)
        assert c * c == pytest.approx((pp - pm) / (2 * h), rel=1e-5), comp


@pytest.mark.parametrize("law", LAWS)
def test_oracle_uniform_state_and_conservation(law):
    mesh, t = amr_mesh(dim=2, b=8, nref=3, seed=3)
    p = mg_params(t, law)
    # a uniform state stays uniform bit for bit across the AMR levels
    U = mg_state(mesh, t, p)
    U[: t.n_owned] = U[0:1, :, 0:1]
    o = orc.Oracle(t, p)
    out, _ = o.run(U, 4)
    assert np.array_equal(out[: t.n_owned], U[: t.n_owned])
    # per-material mass and total energy conserved on the periodic mesh
    from godunov_five_eq_gb300.metrics import material_masses

    U = mg_state(mesh, t, p, seed=1)
    out, _ = o.run(U, 10)
    assert np.all(np.isfinite(out[: t.n_owned]))
    m0, m1 = material_masses(t, U), material_masses(t, out)
    assert np.all(np.abs(m1 - m0) <= 1e-13 * np.abs(m0))
    vol = np.asarray(t.level_dx)[t.level[: t.n_owned]] ** 2
    e0 = float(np.sum(U[: t.n_owned, 1].sum(axis=1) * vol))
    e1 = float(np.sum(out[: t.n_owned, 1].sum(axis=1) * vol))
    assert abs(e1 - e0) <= 1e-12 * abs(e0)


def test_mg_params_rejected_when_invalid():
    from godunov_five_eq_gb300.implem import G5Error, GodunovImplemGB300

    mesh, t = amr_mesh(dim=2, b=8, nref=1)
    p = mg_params(t, "jwl")
    bad = configs.HydroParams(**{**p.__dict__, "mg": ((0.0,) * 8, p.mg[1])})  # rho0 = 0
    with pytest.raises(G5Error):
        GodunovImplemGB300(bad, t)
    bad = configs.HydroParams(**{**p.__dict__, "eos": (7, 0)})
    with pytest.raises(G5Error):
        GodunovImplemGB300(bad, t)


# ---------------------------------------------------------------------- GPU
def _gpu_cases():
    out = []
    for law in LAWS:
        mesh, t = amr_mesh(dim=2, b=8, nref=3, seed=5)
        p = mg_params(t, law)
        out.append((f"amr_periodic_{law}", t, p, mg_state(mesh, t, p, seed=2)))
    mesh, t = amr_mesh(dim=2, b=8, nref=3, seed=6, periodic=False)
    p = mg_params(t, "jwl", "air", source_term=1, thinc=1, bc=(2, 2, 3, 3, 1, 1))
    out.append(("amr_walls_jwl_air_mp_thinc", t, p, mg_state(mesh, t, p, seed=3)))
    mesh, t, p, U = configs.mg_shock_tube("shockwave2", "shockwave")
    out.append(("shock_tube_sw2_sw_16", t, p, U))
    mesh, t = amr_mesh(dim=3, b=8, nref=2, seed=7)
    p = mg_params(t, "jwl", "shockwave2", dim=3)
    out.append(("amr_periodic_3d_jwl_sw2", t, p, mg_state(mesh, t, p, seed=4)))
    return out


GPU_CASES = _gpu_cases()


@pytest.mark.gpu
@pytest.mark.parametrize("name,t,p,U", GPU_CASES, ids=[c[0] for c in GPU_CASES])
def test_gpu_fp64_run_bit_exact(name, t, p, U):
    torch = pytest.importorskip("torch")
    from godunov_five_eq_gb300.implem import GodunovImplemGB300

    nsteps = 6
    ref, dts = orc.Oracle(t, p).run(U, nsteps)
    impl = GodunovImplemGB300(p, t)
    d_U = torch.from_numpy(U.copy()).cuda()
    d_U2 = torch.zeros_like(d_U)
    hist = torch.zeros(nsteps * t.n_inst, dtype=torch.float64, device="cuda")
    impl.run(d_U, d_U2, nsteps, mode="fp64", dt_hist=hist)
    torch.cuda.synchronize()
    assert impl.status() == 0
    assert np.array_equal(hist.cpu().numpy(), dts.reshape(-1))
    got = d_U.cpu().numpy()[: t.n_owned]
    diff = np.argwhere(got != ref[: t.n_owned])
    assert diff.size == 0, f"{len(diff)} values differ, first {diff[:5]}"
    # derived pressure and sound speed through the same laws
    for q in ("THERMAL_PRESSURE", "SPEED_OF_SOUND"):
        dq = impl.derived_quantity(d_U, q)
        torch.cuda.synchronize()
        assert np.array_equal(dq.cpu().numpy()[: t.n_owned], orc.derived(p, d_U.cpu().numpy(), q)[: t.n_owned])


@pytest.mark.gpu
@pytest.mark.parametrize("name,t,p,U", GPU_CASES, ids=[c[0] for c in GPU_CASES])
def test_gpu_mixed_mg_laws_l1(name, t, p, U):
    """The FP32-bulk form with the Mie-Grueneisen laws (FP32 laws and mixture
    rules, the pressure numerator rho e - PI in FP64): volume-weighted relative
    L1 <= 1e-5 per conservative variable against the FP64 oracle, per-material
    mass conserved to FP64 round-off."""
    torch = pytest.importorskip("torch")
    from godunov_five_eq_gb300.implem import GodunovImplemGB300
    from godunov_five_eq_gb300.metrics import l1_relative, material_masses

    nsteps = 6
    ref, _ = orc.Oracle(t, p).run(U, nsteps)
    impl = GodunovImplemGB300(p, t)
    d_U = torch.from_numpy(U.copy()).cuda()
    d_U2 = torch.zeros_like(d_U)
    impl.run(d_U, d_U2, nsteps, mode="mixed")
    torch.cuda.synchronize()
    assert impl.status() == 0
    got = d_U.cpu().numpy()
    assert np.all(np.isfinite(got[: t.n_owned]))
    err = l1_relative(t, got, ref)
    assert err.max() <= 1e-5, err
    if all(x == 1 for x in p.bc[: t.dim * 2]):  # periodic: nothing leaves the domain
        m0, m1 = material_masses(t, U), material_masses(t, got)
        assert np.allclose(m1, m0, rtol=1e-12, atol=0)
