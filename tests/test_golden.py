"""Pin the CPU oracle to the reference's own code through golden vectors.

tests/golden/hllc_prim_golden.npz was produced by tests/golden/make_golden.py
from the reference's models/RiemannSolvers.h (riemann_hllc) and
models/utils.h (computePrimitives, hydro_sanitizer) compiled in place with
shim headers.  The oracle must reproduce every value bit for bit.
"""
import ctypes
import os

import numpy as np
import pytest

from oracle.oracle import G5OParams, lib

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "hllc_prim_golden.npz")


def _params(dim, prm):
    p = G5OParams()
    p.dim = dim
    p.b = 8
    p.gamma[0], p.gamma[1], p.pinf[0], p.pinf[1] = prm[0], prm[1], prm[2], prm[3]
    p.smallr, p.smallc = prm[4], prm[5]
    p.slope_type = 1.0
    return p


@pytest.mark.parametrize("dim", [2, 3])
def test_oracle_hllc_matches_reference(dim):
    g = np.load(GOLDEN)
    prm, ql, qr, ref = g[f"d{dim}_prm"], g[f"d{dim}_ql"], g[f"d{dim}_qr"], g[f"d{dim}_hllc"]
    nv = 8 if dim == 2 else 9
    hc = 4 if dim == 2 else 5
    vp = ctypes.c_void_p
    bad = 0
    for i in range(len(prm)):
        p = _params(dim, prm[i])
        a, b = np.ascontiguousarray(ql[i]), np.ascontiguousarray(qr[i])
        out = np.zeros(nv + 3)
        lib().g5o_riemann_hllc(ctypes.byref(p), a.ctypes.data_as(vp), b.ctypes.data_as(vp), out.ctypes.data_as(vp))
        out[hc] = out[hc + 2] = 0.0  # flux volume-fraction entries are set by the caller, not by riemann_hllc
        same = (out == ref[i]) | (np.isnan(out) & np.isnan(ref[i]))
        bad += int(not same.all())
    assert bad == 0, f"{bad} of {len(prm)} HLLC cases differ"


@pytest.mark.parametrize("dim", [2, 3])
def test_oracle_primitives_match_reference(dim):
    g = np.load(GOLDEN)
    prm, u, qref, cref = g[f"d{dim}_prm"], g[f"d{dim}_u"], g[f"d{dim}_q"], g[f"d{dim}_c"]
    nv = 8 if dim == 2 else 9
    vp = ctypes.c_void_p
    bad = 0
    for i in range(len(prm)):
        p = _params(dim, prm[i])
        a = np.ascontiguousarray(u[i])
        q = np.zeros(nv)
        c = lib().g5o_compute_primitives(ctypes.byref(p), a.ctypes.data_as(vp), q.ctypes.data_as(vp))
        same = np.all((q == qref[i]) | (np.isnan(q) & np.isnan(qref[i]))) and (c == cref[i] or (np.isnan(c) and np.isnan(cref[i])))
        bad += int(not same)
    assert bad == 0, f"{bad} of {len(prm)} primitive conversions differ"


def test_golden_vectors_cover_all_hllc_waves():
    """The states exercise the four sampled regions of the HLLC fan."""
    g = np.load(GOLDEN)
    seen = set()
    for dim in (2, 3):
        ql, qr, out = g[f"d{dim}_ql"], g[f"d{dim}_qr"], g[f"d{dim}_hllc"]
        nv = 8 if dim == 2 else 9
        us = out[:, nv]
        ul, ur = ql[:, 2], qr[:, 2]
        seen |= {"left"} if np.any(us == ul) else set()
        seen |= {"right"} if np.any(us == ur) else set()
        seen |= {"star_left"} if np.any((us > 0) & (us != ul)) else set()
        seen |= {"star_right"} if np.any((us <= 0) & (us != ur)) else set()
    assert seen == {"left", "right", "star_left", "star_right"}


# ---------------------------------------------------------------------------
# One whole block timestep (slopes, MUSCL-Hancock / THINC reconstruction,
# HLLC fluxes with their dt/dx scaling, per-direction read-back update with
# the volume-fraction source term, renormalisation, CFL reduction) against the
# reference's own scheme functors, on periodic tiles of same-level blocks.
# tests/golden/scheme_step_golden.npz comes from tests/golden/make_scheme_golden.py.
# ---------------------------------------------------------------------------
SCHEME_GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "scheme_step_golden.npz")
REFPIN_LIB = os.path.join(os.path.dirname(os.path.dirname(__file__)), "oracle", "_ref", "librefpin.so")


def _scheme_cases():
    g = np.load(SCHEME_GOLDEN)
    return sorted({k.split("/")[0] for k in g.keys()})


def _tile(dim, b, nb, prm):
    from godunov_five_eq_gb300 import configs
    from godunov_five_eq_gb300.mesh import BlockMesh

    mesh = BlockMesh(dim, b, (nb,) * dim, (True,) * dim, 0, 0, scaling=1.0)
    t = mesh.build()
    p = configs.HydroParams(
        dim=dim,
        bsize=b,
        gamma=(prm[0], prm[1]),
        pinf=(prm[2], prm[3]),
        smallr=prm[4],
        smallc=prm[5],
        slope_type=prm[6],
        cfl=0.4,
        thinc=int(prm[7]),
        thinc_beta=prm[8],
        thinc_eps=prm[9],
        integrator=int(prm[10]),
        source_term=int(prm[11]),
        bc=(1,) * 6,
        level_dx=t.level_dx,
    )
    return mesh, t, p


def _oracle_step(t, p, U, dt):
    from oracle.oracle import Oracle

    o = Oracle(t, p)
    U = np.ascontiguousarray(U)
    o.fill_outside(U)
    out = o.step(U, dt)
    o.fill_outside(out)
    inv = float(o.inv_dt(out)[0])
    o.close()
    return out[: t.n_owned], inv


@pytest.mark.parametrize("name", _scheme_cases())
def test_oracle_scheme_step_matches_reference_golden(name):
    import dataclasses

    g = np.load(SCHEME_GOLDEN)
    prm, (dim, b, nb), dt = g[f"{name}/prm"], g[f"{name}/shape"], float(g[f"{name}/dt"][0])
    mesh, t, p = _tile(int(dim), int(b), int(nb), prm)
    U = np.zeros((t.n_total, t.nv, t.ncell))
    U[: t.n_owned] = g[f"{name}/U"]
    got, inv = _oracle_step(t, p, U, dt)
    ref = g[f"{name}/U2"]
    assert np.array_equal(got, ref), f"{(got != ref).sum()} of {ref.size} values differ"
    assert inv == float(g[f"{name}/inv_dt"][0])
    if p.thinc:
        # the THINC branch was taken: the MUSCL step gives another state
        plain, _ = _oracle_step(t, dataclasses.replace(p, thinc=0), U, dt)
        assert not np.array_equal(plain, ref)


def test_scheme_golden_cases_cover_the_options():
    g = np.load(SCHEME_GOLDEN)
    opts = {(int(g[f"{n}/shape"][0]), int(g[f"{n}/prm"][7]), int(g[f"{n}/prm"][10]), int(g[f"{n}/prm"][11]), float(g[f"{n}/prm"][6])) for n in _scheme_cases()}
    assert {o[0] for o in opts} == {2, 3}  # 2D and 3D
    assert {o[1] for o in opts} == {0, 1}  # MUSCL and THINC
    assert {o[2] for o in opts} == {0, 1}  # HANCOCK and RK1
    assert {o[3] for o in opts} == {0, 1}  # ALLAIRE_KOKH and MILLER_PUCKETT
    assert {o[4] for o in opts} == {1.0, 2.0}  # minmod and MC


@pytest.mark.skipif(not os.path.exists(REFPIN_LIB), reason="reference-pinning library not built (needs the reference tree)")
@pytest.mark.parametrize("dim", [2, 3])
def test_oracle_scheme_step_matches_reference_live(dim):
    """Fresh states and every option combination against the reference's
    scheme code compiled in this checkout (oracle/_ref/librefpin.so)."""
    from tests.golden.make_scheme_golden import load, params_vector, reference_step, tile_case

    lib = load()
    nb = 2 if dim == 2 else 1
    bad = []
    n = 0
    for mats in ("water_air", "air_helium"):
        for thinc in (0, 1):
            for integ in (0, 1):
                for st in (0, 1):
                    for slope in (1.0, 2.0):
                        seed = 100 + n
                        n += 1
                        mesh, t, p, U = tile_case(dim, 8, nb, mats, thinc, integ, st, slope, seed)
                        from oracle.oracle import Oracle

                        o = Oracle(t, p)
                        dt = float(o.dt(U)[0])
                        o.close()
                        ref, inv_ref = reference_step(lib, dim, 8, nb, params_vector(p, thinc, integ, st), U[: t.n_owned], dt)
                        got, inv = _oracle_step(t, p, U, dt)
                        if not (np.array_equal(got, ref) and inv == inv_ref):
                            bad.append((mats, thinc, integ, st, slope, int((got != ref).sum())))
    assert not bad, bad


# ---------------------------------------------------------------------------
# Refinement flags against the reference's own ComputeRefineFlags (all three
# indicators, swept over the refine / coarsen / Loehner thresholds so that
# every block's largest indicator is pinned to an interval; coarsening allowed
# with level_min -1).  tests/golden/refine_flags_golden.npz comes from
# `python tests/golden/make_scheme_golden.py --flags`.
# ---------------------------------------------------------------------------
FLAGS_GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "refine_flags_golden.npz")


def _oracle_flag_sweep(t, p, U, eps_lohner, eps_refine, eps_coarsen):
    from oracle.oracle import Oracle

    o = Oracle(t, p)
    U = np.ascontiguousarray(U)
    o.fill_outside(U)
    out = np.zeros((3, len(eps_lohner), len(eps_refine), len(eps_coarsen), t.n_owned), np.int8)
    for ind in range(3):
        for a, el in enumerate(eps_lohner):
            for i, er in enumerate(eps_refine):
                for j, ec in enumerate(eps_coarsen):
                    out[ind, a, i, j] = o.refine_flags(U, ind, er, ec, el, -1, 2)
    o.close()
    return out


@pytest.mark.parametrize("seed", [11, 12])
def test_oracle_refine_flags_match_reference_golden(seed):
    from tests.golden.make_scheme_golden import EPS_COARSEN, EPS_LOHNER, EPS_REFINE, flag_tile

    g = np.load(FLAGS_GOLDEN)
    (mesh, t, p, _), nb = flag_tile(2, seed)
    U = np.zeros((t.n_total, t.nv, t.ncell))
    U[: t.n_owned] = g[f"seed{seed}/U"]
    ref = g[f"seed{seed}/flags"]
    got = _oracle_flag_sweep(t, p, U, EPS_LOHNER, EPS_REFINE, EPS_COARSEN)
    assert np.array_equal(got, ref), f"{(got != ref).sum()} of {ref.size} flags differ"
    assert {0, 1, 2} <= set(np.unique(np.concatenate([np.load(FLAGS_GOLDEN)[f"seed{s}/flags"].ravel() for s in (11, 12)])))


@pytest.mark.skipif(not os.path.exists(REFPIN_LIB), reason="reference-pinning library not built (needs the reference tree)")
@pytest.mark.parametrize("dim", [2, 3])
def test_oracle_refine_flags_match_reference_live(dim):
    from tests.golden.make_scheme_golden import EPS_COARSEN, EPS_LOHNER, EPS_REFINE, flag_tile, load_flags, sweep

    lib = load_flags()
    for seed in (21, 22, 23):
        (mesh, t, p, U), nb = flag_tile(dim, seed)
        ref = sweep(lib, dim, nb, U[: t.n_owned])
        got = _oracle_flag_sweep(t, p, U, EPS_LOHNER, EPS_REFINE, EPS_COARSEN)
        assert np.array_equal(got, ref), (seed, int((got != ref).sum()))


# ---------------------------------------------------------------------------
# Boundary fill against the reference's own FillOutsideCellFunctor
# (border_conditions/FillOutside.cpp:44-172) on non-periodic AMR meshes with
# ZERO_GRADIENT and WALL faces.  tests/golden/fill_outside_golden.npz comes from
# `python tests/golden/make_scheme_golden.py --fill`.
# ---------------------------------------------------------------------------
FILL_GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "fill_outside_golden.npz")


def _oracle_fill(t, U, bc):
    from oracle.oracle import Oracle
    from tests.helpers import water_air_params

    p = water_air_params(t, dim=t.dim, b=t.bsize, bc=tuple(bc) + (2,) * (6 - len(bc)))
    o = Oracle(t, p)
    U = np.ascontiguousarray(U).copy()
    o.fill_outside(U)
    o.close()
    return U


def _fill_cases():
    from tests.golden.make_scheme_golden import FILL_CASES

    return sorted(FILL_CASES)


@pytest.mark.parametrize("name", _fill_cases())
def test_oracle_fill_outside_matches_reference_golden(name):
    from tests.golden.make_scheme_golden import FILL_CASES, fill_case

    dim, seed, bc = FILL_CASES[name]
    mesh, t, U = fill_case(dim, seed)
    assert t.n_outside > 0
    ref = np.load(FILL_GOLDEN)[f"{name}/outside"].astype(np.float64)
    got = _oracle_fill(t, U, bc)[t.n_owned :]
    assert np.array_equal(got, ref), f"{(got != ref).sum()} of {ref.size} values differ"
    # every outside value is a copy of an owned value, negated only by a WALL face
    assert np.all(np.abs(ref) >= 1)
    assert (ref < 0).any() == (3 in bc[: 2 * dim])


@pytest.mark.skipif(not os.path.exists(REFPIN_LIB), reason="reference-pinning library not built (needs the reference tree)")
@pytest.mark.parametrize("dim", [2, 3])
def test_oracle_fill_outside_matches_reference_live(dim):
    """Every ZERO_GRADIENT / WALL combination of the faces (2D; a sample in
    3D) on fresh meshes and states against the reference's FillOutside
    compiled in this checkout."""
    import itertools

    from tests.golden.make_scheme_golden import fill_case, load_fill, reference_fill

    lib = load_fill()
    combos = list(itertools.product((2, 3), repeat=2 * dim))
    if dim == 3:
        combos = combos[::7]
    bad = []
    for k, bc in enumerate(combos):
        mesh, t, U = fill_case(dim, 20 + k % 3)
        U[: t.n_owned] = np.random.default_rng(k).standard_normal(U[: t.n_owned].shape)
        ref = reference_fill(lib, t, U, bc)[t.n_owned :]
        got = _oracle_fill(t, U, bc)[t.n_owned :]
        if not np.array_equal(got, ref):
            bad.append((bc, int((got != ref).sum())))
    assert not bad, bad
