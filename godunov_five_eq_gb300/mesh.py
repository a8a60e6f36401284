"""Block-AMR mesh and the block table consumed by the GPU timestep.

The reference obtains its mesh from the external kalypsso core (p4est forest,
``AMRManager``, orchard keys, a device hashmap and ``StencilHelper``).  None of
that exists here, so this module restates the part the timestep needs:

* a forest of square (cubic) trees laid out as a brick ``nbrick`` with
  optional periodicity per direction (``[p4est_connectivity]`` in the decks);
* leaves are ``bsize^dim`` cell blocks identified by ``(level, ix, iy, iz)``
  in global block coordinates at their level;
* 2:1 balance across faces, edges and corners (the reference's stencil code
  assumes at most one level jump between any two touching leaves,
  scheme/ConvertToPrimitivesVariablesFunctor.cpp:884-922);
* outside blocks: every owned leaf that touches a non-periodic domain face
  gets a twin, translated by one block along each outside normal, that
  carries the boundary values (the reference's outside quadrants,
  border_conditions/FillOutside.cpp:71-170);
* a neighbour table with, for each of the ``3^dim`` same-level neighbour
  slots of an owned block, the level relation (-1 coarser, 0 same, +1 finer)
  and the block indices (the coarse block, the same-level block, or the
  ``2^dim`` children of the virtual same-level neighbour, of which only the
  ones touching the block are filled).

Leaves are ordered tree by tree (x fastest) and in Morton order inside a tree.
Owned blocks come first, outside blocks after them, matching the U layout
``[n_blocks][nv][bsize^dim]``.
"""
from __future__ import annotations

import itertools
from dataclasses import dataclass, field

import numpy as np

# boundary condition codes (border_conditions/FillOutside.h:51-55)
BC_NONE, BC_PERIODIC, BC_ZERO_GRADIENT, BC_WALL = 0, 1, 2, 3
BC_NAMES = {"NONE": 0, "PERIODIC": 1, "ZERO_GRADIENT": 2, "WALL": 3}


def _morton(local: np.ndarray, bits: int) -> int:
    """Interleave the bits of the integer coordinates (x lowest)."""
    key = 0
    dim = len(local)
    for bit in range(bits):
        for e in range(dim):
            key |= ((int(local[e]) >> bit) & 1) << (bit * dim + e)
    return key


@dataclass
class BlockTable:
    """Flat arrays describing one mesh (or a batch of independent meshes)."""

    dim: int
    bsize: int
    n_owned: int
    n_outside: int
    level: np.ndarray  # int32 [n_total]
    coord: np.ndarray  # int32 [n_total, 3]
    nbr: np.ndarray  # int32 [n_owned, 3^dim, 2^dim]
    nbr_rel: np.ndarray  # int8  [n_owned, 3^dim]
    out_src: np.ndarray  # int32 [n_outside]
    out_normal: np.ndarray  # int8 [n_outside, 3]
    out_border: np.ndarray  # int8 [n_outside, 6]
    inst: np.ndarray  # int32 [n_total]
    n_inst: int = 1
    level_dx: np.ndarray = field(default_factory=lambda: np.zeros(32))  # float64 [32]

    @property
    def n_total(self) -> int:
        return self.n_owned + self.n_outside

    @property
    def nv(self) -> int:
        return 8 if self.dim == 2 else 9

    @property
    def ncell(self) -> int:
        return self.bsize**self.dim

    def owned_cells(self) -> int:
        return self.n_owned * self.ncell


REMAP_COPY, REMAP_REFINED, REMAP_COARSENED = 0, 1, 2


@dataclass
class RemapTable:
    """Old -> new owned-block map of one mesh adaptation.

    kind[j] = REMAP_COPY: new block j is old block src[j, 0];
    REMAP_REFINED: new block j is child src[j, 1] (x + 2y + 4z) of old block
    src[j, 0]; REMAP_COARSENED: new block j is the parent of the old blocks
    src[j, 0 .. 2^dim - 1] (child order x + 2y + 4z)."""

    dim: int
    bsize: int
    n_old: int
    kind: np.ndarray  # int8 [n_new]
    src: np.ndarray  # int32 [n_new, 2^dim]

    @property
    def n_new(self) -> int:
        return int(self.kind.shape[0])

    def counts(self) -> dict:
        return {name: int((self.kind == v).sum()) for name, v in (("copied", 0), ("refined", 1), ("coarsened", 2))}


class BlockMesh:
    """A balanced block-AMR forest on a brick of trees."""

    def __init__(self, dim, bsize, nbrick, periodic, level_min, level_max, scaling=1.0):
        if dim not in (2, 3):
            raise ValueError("dim must be 2 or 3")
        if bsize < 4 or bsize % 2:
            raise ValueError("block size must be even and >= 4 (2 ghost layers)")
        self.dim = dim
        self.bsize = bsize
        self.nbrick = tuple(int(n) for n in nbrick)[:dim]
        self.periodic = tuple(bool(p) for p in periodic)[:dim]
        self.level_min = int(level_min)
        self.level_max = int(level_max)
        self.scaling = float(scaling)
        self.leaves: set = set()
        L = self.level_min
        ranges = [range(self.nbrick[e] << L) for e in range(dim)]
        for c in itertools.product(*ranges):
            self.leaves.add((L,) + tuple(c) + (0,) * (3 - dim))

    # ------------------------------------------------------------------ geometry
    def extent(self, level: int, e: int) -> int:
        return self.nbrick[e] << level

    def cell_length(self, level: int) -> float:
        """Cell size at a level: (1 / (bsize 2^level)) * scaling_factor
        (compute_cell_length(level, bx) * scaling, ComputeFluxesAndStoreFunctor.cpp:359)."""
        return (1.0 / float(self.bsize << level)) * self.scaling

    def level_dx(self) -> np.ndarray:
        return np.array([self.cell_length(L) for L in range(32)], dtype=np.float64)

    def wrap(self, level, c):
        """Periodic wrap; returns (coords, outside_mask)."""
        out = []
        mask = []
        for e in range(self.dim):
            n = self.extent(level, e)
            v = c[e]
            if self.periodic[e]:
                v %= n
                mask.append(False)
            else:
                mask.append(v < 0 or v >= n)
            out.append(v)
        out += [0] * (3 - self.dim)
        return tuple(out), mask

    # --------------------------------------------------------------- refinement
    def children(self, key):
        L, x, y, z = key
        kids = []
        for cz in range(2 if self.dim == 3 else 1):
            for cy in range(2):
                for cx in range(2):
                    kids.append((L + 1, 2 * x + cx, 2 * y + cy, 2 * z + cz if self.dim == 3 else 0))
        return kids

    def refine(self, keys) -> int:
        n = 0
        for k in keys:
            if k in self.leaves and k[0] < self.level_max:
                self.leaves.remove(k)
                self.leaves.update(self.children(k))
                n += 1
        return n

    def _covering_leaf(self, level, c):
        """Leaf at level <= `level` that contains the same-level position c (inside domain)."""
        for L in range(level, self.level_min - 1, -1):
            s = level - L
            key = (L,) + tuple(ci >> s for ci in c[: self.dim]) + (0,) * (3 - self.dim)
            if key in self.leaves:
                return key
        return None

    def balance(self) -> int:
        """Enforce 2:1 balance across faces, edges and corners."""
        total = 0
        offsets = [o for o in itertools.product((-1, 0, 1), repeat=self.dim) if any(o)]
        while True:
            marked = set()
            for key in self.leaves:
                L = key[0]
                if L - self.level_min < 2:
                    continue
                for o in offsets:
                    c = tuple(key[1 + e] + o[e] for e in range(self.dim))
                    cw, outside = self.wrap(L, c)
                    if any(outside):
                        continue
                    leaf = self._covering_leaf(L, cw)
                    if leaf is not None and leaf[0] < L - 1:
                        marked.add(leaf)
            if not marked:
                return total
            total += self.refine(marked)

    # ------------------------------------------------------------ adaptation
    def _coarsening_breaks_balance(self, parent) -> bool:
        """True when a leaf finer than parent level + 1 touches `parent`
        (faces, edges or corners): some same-level position next to one of
        its children is not covered by a leaf of that level or coarser."""
        L = parent[0] + 1
        lo = [2 * parent[1 + e] for e in range(self.dim)]
        offsets = itertools.product(*[range(lo[e] - 1, lo[e] + 3) for e in range(self.dim)])
        for c in offsets:
            if all(lo[e] <= c[e] < lo[e] + 2 for e in range(self.dim)):
                continue
            cw, outside = self.wrap(L, c)
            if any(outside):
                continue
            if self._covering_leaf(L, cw) is None:
                return True
        return False

    def adapt(self, flags) -> "RemapTable":
        """Apply per-block refine flags and return the old -> new block map.

        `flags` holds one ComputeRefineFlags code per owned block of the
        current table (ordered_leaves order): 2 refine, 0 coarsen, other
        values keep the block (scheme/ComputeRefineFlags.cpp:250-368).  The
        forest adaptation itself is p4est's (the reference's
        AMRManager::rebuild_from_context, SolverGodunovFiveEq.cpp:258-314);
        restated here as: refine every flagged block below level_max,
        restore 2:1 balance by refining, then coarsen each complete family
        of leaves above level_min whose 2^dim members are all flagged 0 and
        were not refined, unless the coarse block would touch a leaf two
        levels finer (such families are kept until none is left).  Every
        new block therefore comes from one old block (kept or refined once)
        or from the 2^dim old children of a family."""
        old = self.ordered_leaves()
        flags = np.asarray(flags).reshape(-1)
        if flags.shape[0] != len(old):
            raise ValueError(f"expected {len(old)} flags, got {flags.shape[0]}")
        old_index = {k: i for i, k in enumerate(old)}
        refined_from: dict = {}

        def refine_one(k):
            if k in refined_from:
                raise RuntimeError("a block would be refined twice in one adaptation")
            self.leaves.remove(k)
            for ch in self.children(k):
                self.leaves.add(ch)
                refined_from[ch] = k

        for k, f in zip(old, flags):
            if f == 2 and k[0] < self.level_max:
                refine_one(k)
        # 2:1 balance by refinement (the same sweep as balance())
        offsets = [o for o in itertools.product((-1, 0, 1), repeat=self.dim) if any(o)]
        while True:
            marked = set()
            for key in self.leaves:
                L = key[0]
                if L - self.level_min < 2:
                    continue
                for o in offsets:
                    c = tuple(key[1 + e] + o[e] for e in range(self.dim))
                    cw, outside = self.wrap(L, c)
                    if any(outside):
                        continue
                    leaf = self._covering_leaf(L, cw)
                    if leaf is not None and leaf[0] < L - 1:
                        marked.add(leaf)
            if not marked:
                break
            for k in marked:
                if k[0] < self.level_max:
                    refine_one(k)
        # coarsening of complete families
        parents = set()
        for k, f in zip(old, flags):
            if f == 0 and k[0] > self.level_min:
                parents.add((k[0] - 1,) + tuple(c >> 1 for c in k[1 : 1 + self.dim]) + (0,) * (3 - self.dim))
        families = {}
        for P in parents:
            kids = self.children(P)
            if all(ch in self.leaves and ch in old_index and flags[old_index[ch]] == 0 for ch in kids):
                families[P] = kids
        for P, kids in families.items():
            self.leaves.difference_update(kids)
            self.leaves.add(P)
        while True:
            undo = [P for P in families if self._coarsening_breaks_balance(P)]
            if not undo:
                break
            for P in undo:
                self.leaves.remove(P)
                self.leaves.update(families.pop(P))
        new = self.ordered_leaves()
        nc = 2**self.dim
        kind = np.zeros(len(new), np.int8)
        src = np.full((len(new), nc), -1, np.int32)
        for j, k in enumerate(new):
            if k in old_index:
                src[j, 0] = old_index[k]
            elif k in refined_from:
                P = refined_from[k]
                kind[j] = REMAP_REFINED
                src[j, 0] = old_index[P]
                src[j, 1] = sum(((k[1 + e] & 1) << e) for e in range(self.dim))
            else:
                kind[j] = REMAP_COARSENED
                src[j, :] = [old_index[ch] for ch in families[k]]
        return RemapTable(dim=self.dim, bsize=self.bsize, n_old=len(old), kind=kind, src=src)

    # ------------------------------------------------------------------ tables
    def ordered_leaves(self):
        Lmax = max(k[0] for k in self.leaves)

        def sort_key(k):
            L = k[0]
            c = np.array(k[1 : 1 + self.dim])
            tree = c >> L
            tidx = int(tree[0]) + self.nbrick[0] * (int(tree[1]) + (self.nbrick[1] * int(tree[2]) if self.dim == 3 else 0))
            local = (c - (tree << L)) << (Lmax - L)
            return (tidx, _morton(local, Lmax))

        return sorted(self.leaves, key=sort_key)

    def build(self) -> BlockTable:
        dim = self.dim
        owned = self.ordered_leaves()
        index = {k: i for i, k in enumerate(owned)}
        # outside twins
        outside = []
        normals = []
        borders = []
        srcs = []
        for i, k in enumerate(owned):
            L = k[0]
            touch = []  # per dim: -1 at min face, +1 at max face, 0 none (non-periodic only)
            border = [0] * 6
            for e in range(dim):
                n = self.extent(L, e)
                lo = k[1 + e] == 0
                hi = k[1 + e] == n - 1
                border[2 * e] = int(lo)
                border[2 * e + 1] = int(hi)
                t = []
                if not self.periodic[e]:
                    if lo:
                        t.append(-1)
                    if hi:
                        t.append(1)
                touch.append(t)
            choices = [[0] + touch[e] for e in range(dim)]
            for nrm in itertools.product(*choices):
                if not any(nrm):
                    continue
                tk = (L,) + tuple(k[1 + e] + nrm[e] for e in range(dim)) + (0,) * (3 - dim)
                outside.append(tk)
                normals.append(list(nrm) + [0] * (3 - dim))
                borders.append(border)
                srcs.append(i)
        n_owned = len(owned)
        for j, k in enumerate(outside):
            index[k] = n_owned + j
        allkeys = owned + outside

        ns = 3**dim
        nc = 2**dim
        nbr = np.full((n_owned, ns, nc), -1, dtype=np.int32)
        rel = np.zeros((n_owned, ns), dtype=np.int8)
        slots = list(itertools.product((-1, 0, 1), repeat=dim))
        for i, k in enumerate(owned):
            L = k[0]
            for d in slots:
                d = d[::-1]  # itertools varies the last entry fastest; slot index has x fastest
                if not any(d):
                    continue
                s = sum((d[e] + 1) * 3**e for e in range(dim))
                c = tuple(k[1 + e] + d[e] for e in range(dim))
                cw, _ = self.wrap(L, c)
                key = (L,) + cw[:dim] + (0,) * (3 - dim)
                if key in index:
                    rel[i, s] = 0
                    nbr[i, s, 0] = index[key]
                    continue
                pkey = (L - 1,) + tuple(cw[e] >> 1 for e in range(dim)) + (0,) * (3 - dim)
                if pkey in index:
                    rel[i, s] = -1
                    nbr[i, s, 0] = index[pkey]
                    continue
                # finer: the children of the virtual neighbour that touch the block
                found = False
                for cidx in range(nc):
                    ch = [(cidx >> e) & 1 for e in range(dim)]
                    if any((d[e] == -1 and ch[e] != 1) or (d[e] == 1 and ch[e] != 0) for e in range(dim)):
                        continue
                    ckey = (L + 1,) + tuple(2 * cw[e] + ch[e] for e in range(dim)) + (0,) * (3 - dim)
                    if ckey not in index:
                        raise RuntimeError(f"mesh not 2:1 balanced around block {k} slot {d}")
                    nbr[i, s, cidx] = index[ckey]
                    found = True
                if not found:
                    raise RuntimeError(f"no neighbour for block {k} slot {d}")
                rel[i, s] = 1
        n_outside = len(outside)
        level = np.array([k[0] for k in allkeys], dtype=np.int32)
        coord = np.array([k[1:4] for k in allkeys], dtype=np.int32).reshape(-1, 3)
        return BlockTable(
            dim=dim,
            bsize=self.bsize,
            n_owned=n_owned,
            n_outside=n_outside,
            level=level,
            coord=coord,
            nbr=nbr,
            nbr_rel=rel,
            out_src=np.array(srcs, dtype=np.int32),
            out_normal=np.array(normals, dtype=np.int8).reshape(-1, 3),
            out_border=np.array(borders, dtype=np.int8).reshape(-1, 6),
            inst=np.zeros(n_owned + n_outside, dtype=np.int32),
            n_inst=1,
            level_dx=self.level_dx(),
        )


def concat_tables(tables: list[BlockTable]) -> BlockTable:
    """Batch independent meshes (instances) into one table.

    Owned blocks of all instances come first (instance by instance), then all
    outside blocks.  Each block records its instance id so that the timestep
    uses a per-instance dt.  All instances must share dim, block size and the
    level -> cell length table.
    """
    dim, b = tables[0].dim, tables[0].bsize
    for t in tables:
        if t.dim != dim or t.bsize != b:
            raise ValueError("instances must share dim and block size")
        if not np.array_equal(t.level_dx, tables[0].level_dx):
            raise ValueError("instances must share the level -> dx table")
    n_owned = sum(t.n_owned for t in tables)
    owned_off = np.cumsum([0] + [t.n_owned for t in tables])
    out_off = n_owned + np.cumsum([0] + [t.n_outside for t in tables])

    def remap(t, i, arr):
        a = arr.copy()
        own = a >= 0
        a[own & (arr < t.n_owned)] += owned_off[i]
        a[own & (arr >= t.n_owned)] += out_off[i] - t.n_owned
        return a

    level = np.concatenate([t.level[: t.n_owned] for t in tables] + [t.level[t.n_owned :] for t in tables])
    coord = np.concatenate([t.coord[: t.n_owned] for t in tables] + [t.coord[t.n_owned :] for t in tables])
    nbr = np.concatenate([remap(t, i, t.nbr) for i, t in enumerate(tables)])
    rel = np.concatenate([t.nbr_rel for t in tables])
    out_src = np.concatenate([t.out_src + owned_off[i] for i, t in enumerate(tables)]).astype(np.int32)
    out_normal = np.concatenate([t.out_normal for t in tables])
    out_border = np.concatenate([t.out_border for t in tables])
    inst = np.concatenate(
        [np.full(t.n_owned, i, np.int32) for i, t in enumerate(tables)]
        + [np.full(t.n_outside, i, np.int32) for i, t in enumerate(tables)]
    )
    return BlockTable(
        dim=dim,
        bsize=b,
        n_owned=n_owned,
        n_outside=int(sum(t.n_outside for t in tables)),
        level=level.astype(np.int32),
        coord=coord.astype(np.int32),
        nbr=nbr.astype(np.int32),
        nbr_rel=rel.astype(np.int8),
        out_src=out_src,
        out_normal=out_normal.astype(np.int8).reshape(-1, 3),
        out_border=out_border.astype(np.int8).reshape(-1, 6),
        inst=inst,
        n_inst=len(tables),
        level_dx=tables[0].level_dx.copy(),
    )


def cell_centers(mesh: BlockMesh, table: BlockTable, blocks=None):
    """Physical cell-centre coordinates, shape [n_blocks, dim, bsize^dim]."""
    b = table.bsize
    dim = table.dim
    blocks = np.arange(table.n_owned) if blocks is None else np.asarray(blocks)
    idx = np.arange(b**dim)
    loc = [idx % b, (idx // b) % b, idx // (b * b)]
    out = np.empty((len(blocks), dim, b**dim))
    for j, n in enumerate(blocks):
        L = table.level[n]
        dx = mesh.cell_length(L)
        for e in range(dim):
            out[j, e] = (table.coord[n, e] * b + loc[e] + 0.5) * dx
    return out
