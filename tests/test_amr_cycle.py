"""Dynamic AMR cycle: host forest adaptation, old -> new block map, remap.

CPU tests check the adaptation (2:1 balance kept, every old block used once,
area conserved) and the oracle remap (conservation, uniform states).  GPU
tests check g5_remap bit for bit against the oracle and a multi-cycle run
(steps + flags + adapt + remap) FP64 bit-exact against the same loop on the
oracle.
"""
import numpy as np
import pytest

from godunov_five_eq_gb300 import configs
from godunov_five_eq_gb300.mesh import REMAP_COARSENED, REMAP_COPY, REMAP_REFINED
from oracle import oracle as orc
from tests.helpers import amr_mesh, smooth_state, water_air_params


def _random_flags(n, seed):
    rng = np.random.default_rng(seed)
    return rng.choice(np.array([0, 1, 2], np.int8), size=n, p=[0.5, 0.3, 0.2])


def _family_flags(mesh, seed):
    """Flags drawn per family (all siblings alike), so that families coarsen."""
    rng = np.random.default_rng(seed)
    draw = {}
    out = []
    for k in mesh.ordered_leaves():
        parent = (k[0] - 1,) + tuple(c >> 1 for c in k[1:])
        if parent not in draw:
            draw[parent] = rng.choice(np.array([0, 1, 2], np.int8), p=[0.5, 0.3, 0.2])
        out.append(draw[parent])
    return np.array(out, np.int8)


def _areas(table):
    return float(np.sum(0.5 ** (table.dim * table.level[: table.n_owned].astype(np.float64))))


@pytest.mark.parametrize("dim,b,periodic,seed", [(2, 8, True, 0), (2, 8, False, 1), (2, 16, True, 2), (3, 8, True, 3), (3, 8, False, 4)])
def test_adapt_map_and_balance(dim, b, periodic, seed):
    mesh, t_old = amr_mesh(dim=dim, b=b, periodic=periodic, seed=seed, nref=3 if dim == 2 else 2)
    old_keys = mesh.ordered_leaves()
    flags = _random_flags(t_old.n_owned, seed) if dim == 2 else _family_flags(mesh, seed)
    rt = mesh.adapt(flags)
    t_new = mesh.build()  # raises when 2:1 balance is broken
    assert rt.n_new == t_new.n_owned and rt.n_old == t_old.n_owned
    assert _areas(t_new) == pytest.approx(_areas(t_old), rel=0, abs=1e-12)
    nch = 2**dim
    used = np.zeros(t_old.n_owned, np.int64)
    refined_children = {}
    for j in range(rt.n_new):
        k, s = rt.kind[j], rt.src[j]
        if k == REMAP_COPY:
            used[s[0]] += 1
            assert t_new.level[j] == t_old.level[s[0]]
        elif k == REMAP_REFINED:
            refined_children.setdefault(int(s[0]), set()).add(int(s[1]))
            assert t_new.level[j] == t_old.level[s[0]] + 1
        else:
            assert k == REMAP_COARSENED
            for c in range(nch):
                used[s[c]] += 1
                assert t_old.level[s[c]] == t_new.level[j] + 1
                assert flags[s[c]] == 0
                # child c of the new block
                key = old_keys[s[c]]
                assert sum(((key[1 + e] & 1) << e) for e in range(dim)) == c
    for parent, kids in refined_children.items():
        assert kids == set(range(nch))
        used[parent] += 1
    assert np.all(used == 1)
    # every block flagged for refinement below level_max was refined
    for i in np.nonzero(flags == 2)[0]:
        if t_old.level[i] < mesh.level_max:
            assert i in refined_children


def test_adapt_noop_and_full_coarsen():
    mesh, t_old = amr_mesh(dim=2, b=8, seed=5)
    rt = mesh.adapt(np.ones(t_old.n_owned, np.int8))
    assert rt.counts() == {"copied": t_old.n_owned, "refined": 0, "coarsened": 0}
    assert np.array_equal(rt.src[:, 0], np.arange(t_old.n_owned))
    # coarsen everything repeatedly: ends at the base level
    for _ in range(4):
        t = mesh.build()
        mesh.adapt(np.zeros(t.n_owned, np.int8))
    t = mesh.build()
    assert np.all(t.level[: t.n_owned] == mesh.level_min)


def _remap_case(dim, b, seed, uniform=False):
    mesh, t_old = amr_mesh(dim=dim, b=b, seed=seed, nref=3 if dim == 2 else 2)
    p = water_air_params(t_old, dim=dim, b=b)
    U = smooth_state(mesh, t_old, p, seed=seed)
    if uniform:
        U[: t_old.n_owned] = U[0:1, :, 0:1]
    rt = mesh.adapt(_family_flags(mesh, seed + 10))
    t_new = mesh.build()
    return mesh, t_old, t_new, p, U, rt


@pytest.mark.parametrize("dim,b", [(2, 8), (3, 8)])
def test_oracle_remap_conserves(dim, b):
    mesh, t_old, t_new, p, U, rt = _remap_case(dim, b, seed=7)
    assert rt.counts()["refined"] > 0 and rt.counts()["coarsened"] > 0
    V = orc.remap(p, rt, U, t_new.n_total)
    ids = configs.ids(dim)

    def total(t, A, v):
        vol = np.asarray(t.level_dx)[t.level[: t.n_owned]] ** dim
        return float(np.sum(A[: t.n_owned, v, :].sum(axis=1) * vol))

    for name in ("IAD0", "IAD1", "IE", "IU", "IA0"):
        a, bb = total(t_old, U, ids[name]), total(t_new, V, ids[name])
        assert abs(a - bb) <= 1e-13 * max(abs(a), 1.0), name
    n = t_new.n_owned
    co = rt.kind == REMAP_COARSENED
    assert np.array_equal(V[:n, ids["IA1"]][co], 1.0 - V[:n, ids["IA0"]][co])
    assert np.array_equal(V[:n, ids["ID"]][co], (V[:n, ids["IAD0"]] + V[:n, ids["IAD1"]])[co])
    # refined blocks: every fine cell is a copy of a parent cell
    for j in np.nonzero(rt.kind == REMAP_REFINED)[0][:4]:
        parent = U[rt.src[j, 0]]
        assert np.all(np.isin(V[j], parent))


def test_oracle_remap_uniform_exact():
    mesh, t_old, t_new, p, U, rt = _remap_case(2, 8, seed=8, uniform=True)
    V = orc.remap(p, rt, U, t_new.n_total)
    ids = configs.ids(2)
    ref = U[0, :, 0]
    for v in range(t_new.nv):
        if v in (ids["ID"], ids["IA1"]):
            continue  # recomputed from the others on coarsened blocks
        assert np.all(V[: t_new.n_owned, v, :] == ref[v]), v


def _cycle_case():
    """Small air-helium shock-bubble on levels 2..4 of a 4x1 brick, 8^2 blocks,
    starting uniformly at level 3 (the first cycle coarsens the smooth regions
    and refines the shock and the bubble edge)."""
    mesh, t, p, U = configs.shock_bubble(level_min=2, level_max=4, bsize=8, initial_level=3)
    return mesh, t, p, U


# SIMPLE_GRADIENT thresholds of the decks
EPS_R, EPS_C = 0.1, 0.0125


def test_oracle_dynamic_cycles_run():
    mesh, t, p, U = _cycle_case()
    o = orc.Oracle(t, p)
    levels_seen = set()
    changed = 0
    for cycle in range(5):
        U, _ = o.run(U, 5)
        f = o.refine_flags(U, 0, EPS_R, EPS_C, 0.02, mesh.level_min, mesh.level_max)
        rt = mesh.adapt(f)
        changed += int(np.any(rt.kind != REMAP_COPY))
        t = mesh.build()
        U = orc.remap(p, rt, U, t.n_total)
        o.close()
        o = orc.Oracle(t, p)
        o.fill_outside(U)
        levels_seen.update(np.unique(t.level[: t.n_owned]).tolist())
        assert np.all(np.isfinite(U))
    assert levels_seen <= {2, 3, 4}
    assert changed > 0


# ----------------------------------------------------------------- GPU side
@pytest.mark.gpu
@pytest.mark.parametrize("dim,b,seed", [(2, 8, 7), (2, 16, 9), (3, 8, 11)])
def test_gpu_remap_bit_exact(dim, b, seed):
    torch = pytest.importorskip("torch")
    from godunov_five_eq_gb300.implem import GodunovImplemGB300

    mesh, t_old, t_new, p, U, rt = _remap_case(dim, b, seed=seed)
    V = orc.remap(p, rt, U, t_new.n_total)
    impl = GodunovImplemGB300(p, t_old)
    d_U = torch.from_numpy(U).cuda()
    d_V = torch.zeros((t_new.n_total, t_new.nv, t_new.ncell), dtype=torch.float64, device="cuda")
    impl.remap(rt, d_U, d_V)
    torch.cuda.synchronize()
    n = t_new.n_owned
    assert np.array_equal(d_V.cpu().numpy()[:n], V[:n])


@pytest.mark.gpu
def test_gpu_remap_rejects_bad_map():
    torch = pytest.importorskip("torch")
    from godunov_five_eq_gb300.implem import G5Error, GodunovImplemGB300

    mesh, t_old, t_new, p, U, rt = _remap_case(2, 8, seed=7)
    impl = GodunovImplemGB300(p, t_old)
    d_U = torch.from_numpy(U).cuda()
    d_V = torch.zeros((t_new.n_total, t_new.nv, t_new.ncell), dtype=torch.float64, device="cuda")
    bad = type(rt)(dim=rt.dim, bsize=rt.bsize, n_old=rt.n_old, kind=rt.kind.copy(), src=rt.src.copy())
    bad.src[0, 0] = rt.n_old  # one past the old blocks
    with pytest.raises(G5Error):
        impl.remap(bad, d_U, d_V)
    bad = type(rt)(dim=rt.dim, bsize=rt.bsize, n_old=rt.n_old, kind=rt.kind.copy(), src=rt.src.copy())
    bad.kind[0] = 3
    with pytest.raises(G5Error):
        impl.remap(bad, d_U, d_V)


@pytest.mark.gpu
def test_gpu_dynamic_amr_cycles_bit_exact():
    """5 AMR cycles of 5 steps each: GPU flags -> host adapt -> GPU remap ->
    new table, against the oracle running the same loop (FP64, bit-exact)."""
    torch = pytest.importorskip("torch")
    from godunov_five_eq_gb300.implem import GodunovImplemGB300

    mesh_g, t, p, U0 = _cycle_case()
    mesh_o, _, _, _ = _cycle_case()
    o = orc.Oracle(t, p)
    impl = GodunovImplemGB300(p, t)
    A = torch.from_numpy(U0).cuda()
    Uo = U0.copy()
    changed = 0
    for cycle in range(5):
        B = torch.empty_like(A)
        impl.begin(A)
        for _ in range(5):
            impl.advance(A, B)
            A, B = B, A
        Uo, _ = o.run(Uo, 5)
        A, t_g, rt_g = impl.do_amr_cycle(mesh_g, A, 0, EPS_R, EPS_C, 0.02)
        f = o.refine_flags(Uo, 0, EPS_R, EPS_C, 0.02, mesh_o.level_min, mesh_o.level_max)
        rt_o = mesh_o.adapt(f)
        t_o = mesh_o.build()
        assert np.array_equal(rt_g.kind, rt_o.kind) and np.array_equal(rt_g.src, rt_o.src)
        changed += int(np.any(rt_o.kind != REMAP_COPY))
        Uo = orc.remap(p, rt_o, Uo, t_o.n_total)
        o.close()
        o = orc.Oracle(t_o, p)
        o.fill_outside(Uo)
        torch.cuda.synchronize()
        assert np.array_equal(A.cpu().numpy(), Uo), f"cycle {cycle}"
    assert changed > 0
    assert impl.status() == 0
