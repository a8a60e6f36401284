"""The native block forest (libg5gpu.so, g5_forest_*) against the Python
restatement of the same algorithms (oracle/forest_py.py): identical leaves,
leaf order, old -> new block maps and block tables over random refinement,
balance and adaptation cycles, in 2D and 3D, periodic and bounded.  Host
code only (no GPU)."""
import numpy as np
import pytest

from godunov_five_eq_gb300.mesh import BlockMesh
from oracle.forest_py import PyBlockMesh

TABLE_FIELDS = ("level", "coord", "nbr", "nbr_rel", "out_src", "out_normal", "out_border")


def _pair(dim, b, nbrick, periodic, lmin, lmax):
    args = (dim, b, nbrick[:dim], (periodic,) * dim, lmin, lmax)
    return BlockMesh(*args), PyBlockMesh(*args)


def _same_tables(a, b):
    ta, tb = a.build(), b.build()
    assert (ta.n_owned, ta.n_outside) == (tb.n_owned, tb.n_outside)
    for name in TABLE_FIELDS:
        assert np.array_equal(getattr(ta, name), getattr(tb, name)), name


CASES = [
    (2, 8, (2, 2, 1), True, 1, 4, 0),
    (2, 16, (4, 1, 1), False, 2, 5, 1),
    (2, 8, (3, 2, 1), False, 0, 4, 2),
    (3, 8, (2, 1, 1), True, 1, 3, 3),
    (3, 8, (2, 2, 2), False, 0, 3, 4),
    # level grids too large for the dense lookup: the hash-map path
    (3, 8, (1, 1, 1), False, 0, 20, 5),
    (2, 16, (2, 1, 1), True, 0, 24, 6),
]


@pytest.mark.parametrize("dim,b,nbrick,periodic,lmin,lmax,seed", CASES)
def test_native_forest_matches_restatement(dim, b, nbrick, periodic, lmin, lmax, seed):
    rng = np.random.default_rng(seed)
    nat, py = _pair(dim, b, nbrick, periodic, lmin, lmax)
    for _ in range(min(lmax - lmin, 4)):
        leaves = sorted(nat.leaves)
        pick = rng.choice(len(leaves), size=min(4, len(leaves)), replace=False)
        keys = [leaves[i] for i in pick]
        assert nat.refine(keys) == py.refine(keys)
        nat.balance()
        py.balance()
        assert nat.leaves == py.leaves
    assert nat.ordered_leaves() == py.ordered_leaves()
    _same_tables(nat, py)
    for cycle in range(4):
        n = len(nat.leaves)
        if cycle % 2 == 0:
            flags = rng.choice(np.array([0, 1, 2], np.int8), size=n, p=[0.5, 0.3, 0.2])
        else:  # per family, so that families coarsen
            draw, flags = {}, []
            for k in nat.ordered_leaves():
                parent = (k[0] - 1,) + tuple(c >> 1 for c in k[1:])
                draw.setdefault(parent, rng.choice(np.array([0, 1, 2], np.int8), p=[0.6, 0.2, 0.2]))
                flags.append(draw[parent])
            flags = np.array(flags, np.int8)
        ra, rb = nat.adapt(flags), py.adapt(flags)
        assert nat.leaves == py.leaves
        assert np.array_equal(ra.kind, rb.kind) and np.array_equal(ra.src, rb.src)
        assert nat.ordered_leaves() == py.ordered_leaves()
        _same_tables(nat, py)


def test_native_forest_rejects_bad_input():
    nat = BlockMesh(2, 8, (2, 2), (True, True), 1, 3)
    with pytest.raises(ValueError):
        nat.adapt(np.ones(3, np.int8))  # wrong flag count
    nat.leaves.add((1, 99, 0, 0))  # outside the brick
    with pytest.raises(RuntimeError):
        nat.build()
    # leaves that do not tile the brick: a parent beside its child, a hole
    nat = BlockMesh(2, 8, (2, 2), (True, True), 1, 3)
    nat.refine([(1, 0, 0, 0)])
    nat.leaves.add((1, 0, 0, 0))
    with pytest.raises(RuntimeError):
        nat.build()
    nat = BlockMesh(2, 8, (2, 2), (True, True), 1, 3)
    nat.leaves.discard((1, 3, 3, 0))
    with pytest.raises(RuntimeError):
        nat.build()
