"""The CPU oracle against the invariants of the method (no GPU).

The reference ships no tests or golden vectors for this path; these are the
exact properties the scheme must satisfy: uniform states are preserved to the
last bit (across AMR levels too), per-material mass, momentum and energy are
conserved to round-off on periodic meshes (refluxing at coarse/fine faces),
and the 2D scheme is symmetric under x<->y exchange.
"""
import numpy as np
import pytest

from godunov_five_eq_gb300 import configs
from godunov_five_eq_gb300.mesh import BlockMesh
from oracle.oracle import Oracle
from tests.helpers import BC_PERIODIC, amr_mesh, smooth_state, water_air_params


def _totals(table, U, names):
    I = configs.ids(table.dim)
    vol = table.level_dx[table.level[: table.n_owned]] ** table.dim
    return np.array([(U[: table.n_owned, I[n]].sum(axis=1) * vol).sum() for n in names])


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("thinc,source_term", [(0, 0), (1, 0), (0, 1)])
def test_uniform_state_preserved(dim, thinc, source_term):
    mesh, t = amr_mesh(dim=dim, b=4 if dim == 3 else 8, nref=2)
    p = water_air_params(t, dim=dim, b=t.bsize, thinc=thinc, source_term=source_term)
    vel = (10.0, -3.0) if dim == 2 else (10.0, -3.0, 2.0)
    U = np.zeros((t.n_total, t.nv, t.ncell))
    U[: t.n_owned] = np.moveaxis(configs.prim_to_cons(dim, p, np.full((t.n_owned, t.ncell), 0.3), 300.0, 0.7, 1e5, vel), 0, 1)
    o = Oracle(t, p)
    U2 = o.step(U, o.dt(U))
    assert np.array_equal(U2[: t.n_owned], U[: t.n_owned])


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("thinc", [0, 1])
def test_conservation_periodic_amr(dim, thinc):
    mesh, t = amr_mesh(dim=dim, b=4 if dim == 3 else 8, nref=3 if dim == 2 else 2)
    assert len(set(t.level[: t.n_owned])) >= 2
    p = water_air_params(t, dim=dim, b=t.bsize, thinc=thinc)
    U = smooth_state(mesh, t, p)
    o = Oracle(t, p)
    names = ["IAD0", "IAD1", "IE", "IU", "IV"] + (["IW"] if dim == 3 else [])
    before = _totals(t, U, names)
    U2 = U
    for _ in range(5):
        U2 = o.step(U2, o.dt(U2))
    after = _totals(t, U2, names)
    scale = np.abs(before) + np.abs(_totals(t, np.abs(U), names))
    assert np.all(np.abs(after - before) <= 1e-13 * scale)
    assert np.all(np.isfinite(U2))


def test_xy_symmetry_2d():
    mesh = BlockMesh(2, 8, (2, 2), (True, True), 1, 1)
    t = mesh.build()
    p = water_air_params(t)
    xc = configs.cell_centers(mesh, t)
    x, y = xc[:, 0], xc[:, 1]
    r = np.sqrt((x - 0.5) ** 2 + (y - 0.5) ** 2)
    a0 = 1e-6 + (1 - 2e-6) * 0.5 * (1 - np.tanh((r - 0.25) / 0.02))
    U = np.zeros((t.n_total, 8, 64))
    U[: t.n_owned] = np.moveaxis(configs.prim_to_cons(2, p, a0, a0 * 1000, (1 - a0) * 1.0, 1e5 + 1e4 * np.exp(-r * r / 0.01), (0 * x, 0 * x)), 0, 1)
    o = Oracle(t, p)
    U2 = U
    for _ in range(3):
        U2 = o.step(U2, o.dt(U2))

    def to_grid(A, v):
        G = np.zeros((32, 32))
        for n in range(t.n_owned):
            bx, by = t.coord[n, 0], t.coord[n, 1]
            G[by * 8 : by * 8 + 8, bx * 8 : bx * 8 + 8] = A[n, v].reshape(8, 8)
        return G

    I = configs.ids(2)
    for v in ["ID", "IE", "IAD0", "IAD1", "IA0"]:
        G = to_grid(U2, I[v])
        assert np.allclose(G, G.T, rtol=1e-12, atol=0)
    assert np.allclose(to_grid(U2, I["IU"]), to_grid(U2, I["IV"]).T, rtol=1e-12, atol=1e-9)


def test_gas_water_runs_and_conserves_materials():
    mesh, t, p, U = configs.gas_water_shock_tube(bsize=8, nx_blocks=16, ny_blocks=2)
    o = Oracle(t, p)
    U2, dts = o.run(U, 20)
    assert np.all(np.isfinite(U2[: t.n_owned]))
    assert np.all(dts > 0)
    # the waves have not reached the x boundaries: partial masses are conserved
    before = _totals(t, U, ["IAD0", "IAD1"])
    after = _totals(t, U2, ["IAD0", "IAD1"])
    assert np.allclose(after, before, rtol=1e-13)


def test_fill_outside_semantics():
    mesh = BlockMesh(2, 4, (2, 1), (False, False), 1, 1)
    t = mesh.build()
    p = water_air_params(t, b=4, bc=(2, 2, 3, 3, 1, 1))
    rng = np.random.default_rng(3)
    U = rng.uniform(1.0, 2.0, size=(t.n_total, 8, 16))
    o = Oracle(t, p)
    o.fill_outside(U)
    I = configs.ids(2)
    for k in range(t.n_outside):
        n = t.n_owned + k
        src = t.out_src[k]
        nrm = t.out_normal[k]
        A = U[n].reshape(8, 4, 4)
        S = U[src].reshape(8, 4, 4)
        if nrm[1] != 0:  # WALL in y is the last face applied
            assert np.array_equal(A[I["IV"]], -S[I["IV"]][::-1, :])
            assert np.array_equal(A[I["IE"]], S[I["IE"]][::-1, :])
        elif nrm[0] == -1:  # ZERO_GRADIENT xmin: copy of the first column
            assert np.array_equal(A[I["IE"]], np.repeat(S[I["IE"]][:, :1], 4, axis=1))
        elif nrm[0] == 1:
            assert np.array_equal(A[I["IE"]], np.repeat(S[I["IE"]][:, -1:], 4, axis=1))


def test_tanh_restatement_accuracy():
    from oracle.oracle import lib

    xs = np.concatenate([np.linspace(-25, 25, 2001), np.logspace(-12, 1, 200)])
    got = np.array([lib().g5o_tanh(float(x)) for x in xs])
    ref = np.tanh(xs)
    assert np.max(np.abs(got - ref) / np.maximum(np.abs(ref), 1e-300)) < 4e-16
