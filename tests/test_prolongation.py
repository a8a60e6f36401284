"""Ghost cells in a coarser neighbour: EXTRAPOLATE_LINEAR_MINMOD and
conservative order-2 / order-4 interpolation
(scheme/ConvertToPrimitivesVariablesFunctor.cpp:893-917).

CPU: the oracle's restatement reproduces linear fields at the fine cell
centres (all three prolongations), and the conservative interpolations keep
the coarse cell's mean over its 2^dim children; invalid combinations are
refused by g5_create before any device call.
GPU: the prolongation pass + step kernels against the oracle, FP64 bit-exact
(g5_step, g5_run, g5_step_host), the FP32-bulk form within its L1 tolerance.
"""
import ctypes
import itertools

import numpy as np
import pytest

from godunov_five_eq_gb300 import implem
from oracle.oracle import Oracle
from tests.helpers import amr_mesh, smooth_state, water_air_params

MINMOD, O2, O4 = 1, 2, 3
L1_TOL_MIXED = 1e-5


def _mesh(dim, b):
    if dim == 2:
        return amr_mesh(dim=2, b=b, nref=4, seed=2, periodic=False)
    return amr_mesh(dim=3, b=b, nref=2, seed=3, periodic=False, nbrick=(2, 1, 1), lmin=1, lmax=2)


def _coarse_ghosts(t):
    """(block, ghost cell) pairs of every ghost cell in a coarser slot."""
    b, dim = t.bsize, t.dim
    for n in range(t.n_owned):
        for g in itertools.product(range(-2, b + 2), repeat=dim):
            d = [(-1 if g[e] < 0 else (1 if g[e] >= b else 0)) for e in range(dim)]
            if not any(d):
                continue
            if t.nbr_rel[n, sum((d[e] + 1) * 3**e for e in range(dim))] < 0:
                yield n, g


def _interpolated_vars(dim):
    ia0 = dim + 2
    return [v for v in range(dim + 6) if v not in (0, ia0 + 2)]  # all but ID and IA1


CPU_CASES = [(2, 8, MINMOD), (2, 8, O2), (2, 8, O4), (2, 16, MINMOD), (2, 16, O2), (2, 16, O4), (3, 8, MINMOD), (3, 8, O2), (3, 8, O4)]


@pytest.mark.parametrize("dim,b,mode", CPU_CASES)
def test_oracle_linear_field_exact(dim, b, mode):
    """Every stencil value of a linear field is the field at the coarse cell
    centre (means of finer cells included), so all three prolongations give
    the field at the fine ghost cell centre."""
    mesh, t = _mesh(dim, b)
    ncell = b**dim
    cells = np.arange(ncell)
    ijk = [(cells // b**e) % b for e in range(dim)]
    dx = t.level_dx[t.level]
    X = [(t.coord[:, e][:, None] * b + ijk[e][None, :] + 0.5) * dx[:, None] for e in range(dim)]
    coefs = np.random.default_rng(0).uniform(-1, 1, size=(t.nv, dim))
    U = np.zeros((t.n_total, t.nv, ncell))
    for v in range(t.nv):
        U[:, v] = 1.0 + sum(coefs[v, e] * X[e] for e in range(dim))
    o = Oracle(t, water_air_params(t, dim=dim, b=b, prolongation=mode))
    vars_ = _interpolated_vars(dim)
    count = 0
    for n, g in _coarse_ghosts(t):
        u = o.ghost_state(U, n, g)
        xc = [(t.coord[n, e] * b + g[e] + 0.5) * dx[n] for e in range(dim)]
        ref = 1.0 + coefs @ np.array(xc)
        assert np.abs(u[vars_] - ref[vars_]).max() < 1e-13
        count += 1
    assert count > 0


@pytest.mark.parametrize("dim,b,mode", [(2, 8, O2), (2, 8, O4), (2, 16, O4), (3, 8, O2), (3, 8, O4)])
def test_oracle_conservative_children_mean(dim, b, mode):
    """The lower and upper half-cell weights average to (0, 1, 0): the mean
    of the 2^dim children of a coarse cell is the coarse cell (which the
    SIMPLE_COPY fill gives every child), on any data."""
    mesh, t = _mesh(dim, b)
    p = water_air_params(t, dim=dim, b=b, prolongation=mode)
    U = smooth_state(mesh, t, p, seed=4)
    o = Oracle(t, p)
    o.fill_outside(U)
    o0 = Oracle(t, water_air_params(t, dim=dim, b=b))
    scale = np.abs(U).max(axis=(0, 2))
    vars_ = _interpolated_vars(dim)
    groups = {}
    for n, g in _coarse_ghosts(t):
        groups.setdefault((n,) + tuple((gi + 2) // 2 for gi in g), []).append(g)
    checked = 0
    for key, gs in groups.items():
        if len(gs) != 2**dim:
            continue
        n = key[0]
        mean = sum(o.ghost_state(U, n, g) for g in gs) / len(gs)
        coarse = o0.ghost_state(U, n, gs[0])
        assert np.all(np.abs(mean[vars_] - coarse[vars_]) <= 1e-14 * scale[vars_])
        checked += 1
    assert checked > 0


def test_invalid_prolongation_rejected_without_device():
    lib = implem.load_library()
    ctx = ctypes.c_void_p()
    p = implem.G5Params()
    p.dim, p.bsize, p.gamma[0], p.gamma[1] = 2, 8, 1.4, 1.4
    p.prolongation = 7
    assert lib.g5_create(ctypes.byref(p), ctypes.byref(ctx)) == -1  # G5_ERR_ARG
    p.prolongation = -1
    assert lib.g5_create(ctypes.byref(p), ctypes.byref(ctx)) == -1


GPU_CASES = CPU_CASES


def _gpu_case(dim, b, mode, thinc=0):
    """The conservative interpolations are not bounded: across the sharp
    interface of the 8-cell 2D mesh the order-2 ghost volume fraction
    overshoots below 0 and the state turns non-physical within three steps
    (the oracle too).  Those cases use the smooth volume-fraction field."""
    mesh, t = _mesh(dim, b)
    bc = (2, 2, 3, 3, 1, 1) if dim == 2 else (2, 2, 3, 3, 2, 3)
    p = water_air_params(t, dim=dim, b=b, bc=bc, prolongation=mode, thinc=thinc)
    sharp = mode == MINMOD or b == 16
    return t, p, smooth_state(mesh, t, p, seed=1, interface=sharp)


@pytest.mark.gpu
@pytest.mark.parametrize("dim,b,mode", GPU_CASES)
def test_gpu_fp64_bit_exact(dim, b, mode):
    torch = pytest.importorskip("torch")
    from godunov_five_eq_gb300.implem import GodunovImplemGB300

    t, p, U = _gpu_case(dim, b, mode, thinc=1 if mode == O2 else 0)
    o = Oracle(t, p)
    nsteps = 3
    ref, dts = o.run(U, nsteps)
    impl = GodunovImplemGB300(p, t)
    d_U = torch.from_numpy(U.copy()).cuda()
    d_U2 = torch.zeros_like(d_U)
    hist = torch.zeros(nsteps * t.n_inst, dtype=torch.float64, device="cuda")
    impl.run(d_U, d_U2, nsteps, mode="fp64", dt_hist=hist)
    torch.cuda.synchronize()
    assert impl.status() == 0
    assert np.array_equal(hist.cpu().numpy(), dts.reshape(-1))
    diff = np.argwhere(d_U.cpu().numpy()[: t.n_owned] != ref[: t.n_owned])
    assert diff.size == 0, f"{len(diff)} values differ, first {diff[:5]}"
    # the prolongation changes the answer (the test would pass vacuously otherwise)
    ref0, _ = Oracle(t, water_air_params(t, dim=dim, b=b, bc=p.bc, thinc=p.thinc)).run(U, nsteps)
    assert not np.array_equal(ref0[: t.n_owned], ref[: t.n_owned])


@pytest.mark.gpu
@pytest.mark.parametrize("dim,b,mode", [(2, 16, O4), (3, 8, MINMOD)])
def test_gpu_host_step_and_mixed(dim, b, mode):
    torch = pytest.importorskip("torch")
    from godunov_five_eq_gb300.implem import GodunovImplemGB300
    from godunov_five_eq_gb300.metrics import l1_relative

    t, p, U = _gpu_case(dim, b, mode)
    o = Oracle(t, p)
    o.fill_outside(U)
    dt = o.dt(U)
    ref = o.step(U, dt)
    impl = GodunovImplemGB300(p, t)
    hU = torch.from_numpy(U.copy()).pin_memory()
    hO = torch.full_like(hU, -7.0).pin_memory()
    impl.do_time_step_host(hU, hO, dt, mode="fp64")
    torch.cuda.synchronize()
    assert impl.status() == 0
    assert np.array_equal(hO.numpy()[: t.n_owned], ref[: t.n_owned])
    nsteps = 5
    refn, _ = o.run(U, nsteps)
    d_U = torch.from_numpy(U.copy()).cuda()
    d_U2 = torch.zeros_like(d_U)
    impl.run(d_U, d_U2, nsteps, mode="mixed")
    torch.cuda.synchronize()
    assert impl.status() == 0
    assert l1_relative(t, d_U.cpu().numpy(), refn).max() <= L1_TOL_MIXED


# ------------------------------------------------- refined blocks of a remap
def _family_flags(mesh, seed):
    rng = np.random.default_rng(seed)
    draw, out = {}, []
    for k in mesh.ordered_leaves():
        parent = (k[0] - 1,) + tuple(c >> 1 for c in k[1:])
        if parent not in draw:
            draw[parent] = rng.choice(np.array([0, 1, 2], np.int8), p=[0.5, 0.3, 0.2])
        out.append(draw[parent])
    return np.array(out, np.int8)


def _refine_case(dim, b, seed, mode, linear=False):
    mesh, t_old = _mesh(dim, b)
    p = water_air_params(t_old, dim=dim, b=b, bc=(2, 2, 3, 3, 2, 3), prolongation=mode)
    o = Oracle(t_old, p)
    if linear:
        ncell = b**dim
        cells = np.arange(ncell)
        ijk = [(cells // b**e) % b for e in range(dim)]
        dx = t_old.level_dx[t_old.level]
        X = [(t_old.coord[:, e][:, None] * b + ijk[e][None, :] + 0.5) * dx[:, None] for e in range(dim)]
        coefs = np.random.default_rng(seed).uniform(-1, 1, size=(t_old.nv, dim))
        U = np.zeros((t_old.n_total, t_old.nv, ncell))
        for v in range(t_old.nv):
            U[:, v] = 1.0 + sum(coefs[v, e] * X[e] for e in range(dim))
    else:
        U = smooth_state(mesh, t_old, p, seed=seed, interface=False)
        o.fill_outside(U)
        coefs = None
    rt = mesh.adapt(_family_flags(mesh, seed + 10))
    t_new = mesh.build()
    return mesh, t_old, t_new, p, o, U, rt, coefs


@pytest.mark.parametrize("dim,b,mode", CPU_CASES)
def test_oracle_refined_blocks_linear_exact(dim, b, mode):
    """Refined blocks of a linear field: every fine cell is the field at its
    centre when no neighbour of the parent is coarser (a coarser neighbour
    gives its stencil points the value of the coarse cell holding them, as
    the ghost fill does, which is first order)."""
    mesh, t_old, t_new, p, o, U, rt, coefs = _refine_case(dim, b, 3, mode, linear=True)
    V = o.remap(rt, U, t_new.n_total)
    ref_idx = [j for j in np.nonzero(rt.kind == 1)[0] if (t_old.nbr_rel[rt.src[j, 0]] >= 0).all()]
    assert len(ref_idx) > 0
    ncell = b**dim
    cells = np.arange(ncell)
    ijk = [(cells // b**e) % b for e in range(dim)]
    vars_ = _interpolated_vars(dim)
    for j in ref_idx:
        dx = t_new.level_dx[t_new.level[j]]
        X = [(t_new.coord[j, e] * b + ijk[e] + 0.5) * dx for e in range(dim)]
        ref = 1.0 + coefs @ np.array(X)
        assert np.abs(V[j][vars_] - ref[vars_]).max() < 1e-13


@pytest.mark.parametrize("dim,b,mode", [(2, 8, O2), (2, 16, O4), (3, 8, O2), (3, 8, O4)])
def test_oracle_refined_blocks_conservative(dim, b, mode):
    """Conservative interpolation: the 2^dim fine cells of a parent cell
    average to it (SIMPLE_COPY refinement gives every fine cell the parent)."""
    mesh, t_old, t_new, p, o, U, rt, _ = _refine_case(dim, b, 4, mode)
    from oracle.oracle import remap as remap_copy

    V = o.remap(rt, U, t_new.n_total)
    V0 = remap_copy(p, rt, U, t_new.n_total)
    scale = np.abs(U).max(axis=(0, 2))
    vars_ = _interpolated_vars(dim)
    ref_idx = np.nonzero(rt.kind == 1)[0]
    assert ref_idx.size > 0
    for j in ref_idx:
        for v in vars_:
            arr = V[j, v].reshape((b,) * dim)  # [z][y][x] or [y][x]
            blocks = arr.reshape(*[m for _ in range(dim) for m in (b // 2, 2)])
            mean = blocks.mean(axis=tuple(range(1, 2 * dim, 2)))
            par = V0[j, v].reshape((b,) * dim)[tuple(slice(0, None, 2) for _ in range(dim))]
            assert np.abs(mean - par).max() <= 1e-14 * scale[v]
    # copied and coarsened blocks are untouched by the prolongation
    other = rt.kind != 1
    assert np.array_equal(V[: t_new.n_owned][other], V0[: t_new.n_owned][other])


@pytest.mark.gpu
@pytest.mark.parametrize("dim,b,mode", GPU_CASES)
def test_gpu_remap_refined_bit_exact(dim, b, mode):
    torch = pytest.importorskip("torch")
    from godunov_five_eq_gb300.implem import GodunovImplemGB300

    mesh, t_old, t_new, p, o, U, rt, _ = _refine_case(dim, b, 7, mode)
    V = o.remap(rt, U, t_new.n_total)
    impl = GodunovImplemGB300(p, t_old)
    d_U = torch.from_numpy(U).cuda()
    d_V = torch.zeros((t_new.n_total, t_new.nv, t_new.ncell), dtype=torch.float64, device="cuda")
    impl.remap(rt, d_U, d_V)
    torch.cuda.synchronize()
    assert impl.status() == 0
    n = t_new.n_owned
    assert np.array_equal(d_V.cpu().numpy()[:n], V[:n])


@pytest.mark.gpu
@pytest.mark.parametrize("mode", [MINMOD, O2])
def test_gpu_amr_cycles_with_prolongation_bit_exact(mode):
    """Three cycles of (5 steps, GPU flags, host adaptation, GPU remap) on
    the 8-cell shock-bubble with a prolongation in the ghost fill and the
    refinement, against the same loop on the oracle (FP64, bit-exact)."""
    torch = pytest.importorskip("torch")
    import dataclasses

    from godunov_five_eq_gb300 import configs
    from godunov_five_eq_gb300.implem import GodunovImplemGB300

    def case():
        mesh, t, p, U = configs.shock_bubble(level_min=2, level_max=4, bsize=8, initial_level=3)
        return mesh, t, dataclasses.replace(p, prolongation=mode), U

    mesh_g, t, p, U0 = case()
    mesh_o, _, _, _ = case()
    o = Oracle(t, p)
    impl = GodunovImplemGB300(p, t)
    A = torch.from_numpy(U0).cuda()
    Uo = U0.copy()
    for cycle in range(3):
        B = torch.empty_like(A)
        impl.begin(A)
        for _ in range(5):
            impl.advance(A, B)
            A, B = B, A
        Uo, _ = o.run(Uo, 5)
        A, t_g, rt_g = impl.do_amr_cycle(mesh_g, A, 0, 0.1, 0.0125, 0.02)
        o.fill_outside(Uo)
        f = o.refine_flags(Uo, 0, 0.1, 0.0125, 0.02, mesh_o.level_min, mesh_o.level_max)
        rt_o = mesh_o.adapt(f)
        t_o = mesh_o.build()
        assert np.array_equal(rt_g.kind, rt_o.kind) and np.array_equal(rt_g.src, rt_o.src)
        Uo = o.remap(rt_o, Uo, t_o.n_total)
        o.close()
        o = Oracle(t_o, p)
        o.fill_outside(Uo)
        torch.cuda.synchronize()
        assert np.array_equal(A.cpu().numpy(), Uo), f"cycle {cycle}"
    assert impl.status() == 0
