"""Derived quantities (ComputeDerivedQuantities, utils/ComputeDerivedQuantities.h).

CPU: the oracle's quantities against their definitions on random states.
GPU: g5_derived_quantity bit-exact against the oracle for all eight
quantities, 2D and 3D, over the requested block range only.
"""
import numpy as np
import pytest

from godunov_five_eq_gb300 import configs
from oracle import oracle as orc
from tests.helpers import amr_mesh, smooth_state, water_air_params

QUANTITIES = orc.DERIVED_QUANTITIES


def _case(dim):
    mesh, t = amr_mesh(dim=dim, b=8, nref=2, seed=dim)
    p = water_air_params(t, dim=dim, b=8)
    return t, p, smooth_state(mesh, t, p, seed=dim)


@pytest.mark.parametrize("dim", [2, 3])
def test_oracle_derived_definitions(dim):
    t, p, U = _case(dim)
    ids = configs.ids(dim)
    n = t.n_owned
    rho = orc.derived(p, U, "RHO_MIX", 0, n)[:n, 0]
    assert np.array_equal(rho, U[:n, ids["ID"]])
    vx = orc.derived(p, U, "VX", 0, n)[:n, 0]
    d = np.maximum(U[:n, ids["ID"]], p.smallr)
    assert np.allclose(vx, U[:n, ids["IU"]] / d, rtol=1e-15, atol=0)
    ek = orc.derived(p, U, "SPECIFIC_EKIN", 0, n)[:n, 0]
    vel2 = (U[:n, ids["IU"]] / d) ** 2 + (U[:n, ids["IV"]] / d) ** 2 + ((U[:n, ids["IW"]] / d) ** 2 if dim == 3 else 0.0)
    assert np.allclose(ek, 0.5 * vel2, rtol=1e-14, atol=0)
    cs = orc.derived(p, U, "SPEED_OF_SOUND", 0, n)[:n, 0]
    mach = orc.derived(p, U, "LOCAL_MACH_NUMBER", 0, n)[:n, 0]
    assert np.allclose(mach * cs, np.sqrt(vel2), rtol=1e-13, atol=1e-12)
    vz = orc.derived(p, U, "VZ", 0, n)[:n, 0]
    if dim == 2:
        assert np.all(vz == 0.0)
    # range: blocks outside [begin, begin + count) stay zero
    part = orc.derived(p, U, "THERMAL_PRESSURE", 3, 5)
    full = orc.derived(p, U, "THERMAL_PRESSURE", 0, n)
    assert np.array_equal(part[3:8], full[3:8]) and np.all(part[:3] == 0) and np.all(part[8:] == 0)


@pytest.mark.gpu
@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("quantity", QUANTITIES)
def test_gpu_derived_bit_exact(dim, quantity):
    torch = pytest.importorskip("torch")
    from godunov_five_eq_gb300.implem import GodunovImplemGB300

    t, p, U = _case(dim)
    impl = GodunovImplemGB300(p, t)
    A = torch.from_numpy(U).cuda()
    ref = orc.derived(p, U, quantity, 2, t.n_owned - 4)
    out = impl.derived_quantity(A, quantity, 2, t.n_owned - 4)
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy(), ref)


@pytest.mark.gpu
def test_gpu_derived_rejects_bad_range():
    torch = pytest.importorskip("torch")
    from godunov_five_eq_gb300.implem import G5Error, GodunovImplemGB300

    t, p, U = _case(2)
    impl = GodunovImplemGB300(p, t)
    A = torch.from_numpy(U).cuda()
    for begin, count in ((-1, 2), (0, t.n_total + 1), (t.n_total, 1)):
        with pytest.raises(G5Error):
            impl.derived_quantity(A, "VX", begin, count)
    with pytest.raises(G5Error):
        impl.derived_quantity(A, 8)
