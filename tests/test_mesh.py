"""Block-AMR mesh builder: balance, neighbour tables, outside blocks (no GPU)."""
import itertools

import numpy as np
import pytest

from godunov_five_eq_gb300.mesh import BlockMesh, concat_tables
from tests.helpers import amr_mesh


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("periodic", [True, False])
def test_balance_and_reciprocity(dim, periodic):
    mesh, t = amr_mesh(dim=dim, b=4, periodic=periodic, nref=3, seed=5)
    ns, nc = 3**dim, 2**dim
    for n in range(t.n_owned):
        for s in range(ns):
            d = [(s // 3**e) % 3 - 1 for e in range(dim)]
            if not any(d):
                continue
            rel = t.nbr_rel[n, s]
            assert rel in (-1, 0, 1)
            if rel == 0:
                m = t.nbr[n, s, 0]
                assert t.level[m] == t.level[n]
                if m < t.n_owned:
                    opp = sum((-d[e] + 1) * 3**e for e in range(dim))
                    assert t.nbr_rel[m, opp] == 0 and t.nbr[m, opp, 0] == n
            elif rel == -1:
                assert t.level[t.nbr[n, s, 0]] == t.level[n] - 1
            else:
                kids = [c for c in t.nbr[n, s] if c >= 0]
                assert kids and all(t.level[c] == t.level[n] + 1 for c in kids)


def test_outside_twins_2d():
    mesh = BlockMesh(2, 4, (2, 1), (False, True), 1, 2)
    mesh.refine([(1, 0, 0, 0)])
    mesh.balance()
    t = mesh.build()
    # every owned block touching x = 0 or x = max has exactly one x-twin; y is periodic
    for k in range(t.n_outside):
        assert t.out_normal[k, 1] == 0
        src = t.out_src[k]
        assert t.level[t.n_owned + k] == t.level[src]
        assert np.array_equal(t.coord[t.n_owned + k, :2], t.coord[src, :2] + t.out_normal[k, :2])


def test_concat_tables_remaps_indices():
    _, a = amr_mesh(dim=2, b=4, nref=2, seed=1, periodic=False)
    _, b = amr_mesh(dim=2, b=4, nref=1, seed=2, periodic=False)
    c = concat_tables([a, b])
    assert c.n_owned == a.n_owned + b.n_owned and c.n_outside == a.n_outside + b.n_outside
    assert c.n_inst == 2
    # instance 1 neighbours stay inside instance 1
    for n in range(a.n_owned, c.n_owned):
        for s in range(9):
            for m in c.nbr[n, s]:
                if m >= 0:
                    assert c.inst[m] == 1
