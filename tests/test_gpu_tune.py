"""g5_tune, the launch-shape autotuner: it searches CTAs per SM, block
claiming, the block walk order and (FP32-bulk 2D with coarse/fine records) the
reflux layout (a separate pass in two layouts, or the step kernel's tail),
keeps the fastest, and every candidate shape gives the same state bit for
bit."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from godunov_five_eq_gb300 import configs  # noqa: E402
from godunov_five_eq_gb300.implem import GodunovImplemGB300  # noqa: E402
from oracle.oracle import oracle_flag_fn  # noqa: E402
from tests.helpers import amr_mesh, smooth_state, water_air_params  # noqa: E402

pytestmark = pytest.mark.gpu


def _run(impl, U, nsteps, mode):
    A = torch.from_numpy(U.copy()).cuda()
    B = torch.zeros_like(A)
    impl.run(A, B, nsteps, mode)
    torch.cuda.synchronize()
    assert impl.status() == 0
    return A.cpu().numpy()


@pytest.mark.parametrize("case", ["shock_bubble_16", "walls_3d_8"])
@pytest.mark.parametrize("mode", ["fp64", "mixed"])
def test_every_tuned_shape_is_bit_identical(case, mode):
    if case == "shock_bubble_16":
        mesh, t, p, U = configs.shock_bubble(level_min=2, level_max=4, flag_fn=oracle_flag_fn())
    else:
        mesh, t = amr_mesh(dim=3, b=8, nref=2, seed=3, periodic=False, nbrick=(2, 1, 1), lmin=1, lmax=2)
        p = water_air_params(t, dim=3, b=8, bc=(2, 2, 3, 3, 2, 3))
        U = smooth_state(mesh, t, p, seed=2)
    assert (t.nbr_rel != 0).any()
    impl = GodunovImplemGB300(p, t)
    ref = _run(impl, U, 3, mode)  # the default shape
    A = torch.from_numpy(U.copy()).cuda()
    impl.fill_outside_quadrants(A)
    B = torch.zeros_like(A)
    choice = impl.tune(A, B, mode)
    assert set(choice) == set(GodunovImplemGB300.SHAPE_KEYS)
    report = impl.tune_report(mode)
    n_layouts = 3 if (mode == "mixed" and t.dim == 2) else 1
    assert len(report) == max(s["ctas_per_sm"] for s, _ in report) * 2 * 2 * n_layouts
    assert all(ms > 0 for _, ms in report)
    n = t.n_owned
    got = _run(impl, U, 3, mode)  # the tuned shape
    assert np.array_equal(got[:n], ref[:n])
    for shape, _ in report:
        impl.set_shape(mode, **shape)
        got = _run(impl, U, 3, mode)
        assert np.array_equal(got[:n], ref[:n]), shape
    impl.close()
