"""Per-material mass conservation on the GPU (both precision forms) and the
mixed form's L-infinity and interface-position errors.

On a periodic 3-level mesh with coarse/fine refluxing nothing enters or
leaves the domain, so sum_cells alpha_k rho_k V must stay constant to FP64
round-off in both forms: the mixed form adds the face fluxes of both
directions as an exact float-float sum with one FP64 add per cell.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from godunov_five_eq_gb300 import configs  # noqa: E402
from godunov_five_eq_gb300.implem import GodunovImplemGB300  # noqa: E402
from godunov_five_eq_gb300.metrics import interface_error, linf_relative, material_masses  # noqa: E402
from oracle.oracle import oracle_flag_fn  # noqa: E402
from tests.helpers import amr_mesh, smooth_state, water_air_params  # noqa: E402

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("mode", ["fp64", "mixed"])
def test_material_mass_conserved(dim, mode):
    mesh, t = amr_mesh(dim=dim, b=8, nref=3 if dim == 2 else 2, seed=1)
    p = water_air_params(t, dim=dim, b=8)
    U = smooth_state(mesh, t, p, seed=1)
    m0 = material_masses(t, U)
    impl = GodunovImplemGB300(p, t)
    A = torch.from_numpy(U).cuda()
    B = torch.zeros_like(A)
    impl.run(A, B, 20, mode=mode)
    torch.cuda.synchronize()
    assert impl.status() == 0
    m1 = material_masses(t, A.cpu().numpy())
    assert np.all(np.abs(m1 - m0) <= 1e-13 * np.abs(m0)), (m0, m1)


def test_mixed_linf_and_interface_position():
    mesh, t, p, U = configs.shock_bubble(level_min=2, level_max=4, bsize=8, flag_fn=oracle_flag_fn())
    outs = {}
    for mode in ("fp64", "mixed"):
        impl = GodunovImplemGB300(p, t)
        A = torch.from_numpy(U.copy()).cuda()
        impl.run(A, torch.zeros_like(A), 60, mode=mode)
        torch.cuda.synchronize()
        outs[mode] = A.cpu().numpy()
    assert linf_relative(t, outs["mixed"], outs["fp64"]).max() < 1e-3
    e = interface_error(t, outs["mixed"], outs["fp64"])
    assert e["volume_rel_diff"] < 1e-3
    assert e["centroid_distance"] < 0.1 * e["finest_dx"]
    assert e["extent_max_shift"] <= e["finest_dx"]
