"""Block-AMR mesh and the block table consumed by the GPU timestep.

The reference obtains its mesh from the external kalypsso core (p4est forest,
``AMRManager``, orchard keys, a device hashmap and ``StencilHelper``).  None of
that exists here, so this module restates the part the timestep needs; the
balance, the adaptation and the table build run in the native forest of
libg5gpu.so (``g5_forest_*``, csrc/g5_forest.cpp):

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
        self._fcache = None  # (native forest, the leaf set it holds or None, leaf count)
        self._leaves: set | None = set()
        L = self.level_min
        ranges = [range(self.nbrick[e] << L) for e in range(dim)]
        for c in itertools.product(*ranges):
            self._leaves.add((L,) + tuple(c) + (0,) * (3 - dim))

    @property
    def leaves(self) -> set:
        """The leaves as a set of (level, x, y, z).  After a native operation
        they live in the native forest until read here.  Change them through
        the methods or by assigning a new set."""
        if self._leaves is None:
            from godunov_five_eq_gb300 import implem

            h = self._fcache[0]
            arr = self._forest_leaves(implem.load_library(), h)
            self._leaves = set(zip(*arr.T.tolist()))
            self._fcache = (h, self._leaves, len(self._leaves))
        return self._leaves

    @leaves.setter
    def leaves(self, value) -> None:
        self.leaves  # noqa: B018  (a forest-only state is read out before it is replaced)
        self._leaves = value

    def _num_leaves(self) -> int:
        return len(self._leaves) if self._leaves is not None else self._fcache[2]

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
        self._drop_forest()
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

    def _forest(self):
        """The native forest (libg5gpu.so) holding the current leaves: the one
        the last native operation left when `leaves` is still the set it
        produced (same object, same size), else a new one from `leaves`."""
        import ctypes

        from godunov_five_eq_gb300 import implem

        lib = implem.load_library()
        cache = self._fcache
        if cache is not None and (self._leaves is None or (cache[1] is self._leaves and cache[2] == len(self._leaves))):
            return lib, cache[0]
        self._drop_forest()
        spec = implem.G5ForestSpec()
        spec.dim, spec.bsize = self.dim, self.bsize
        for e in range(3):
            spec.nbrick[e] = self.nbrick[e] if e < self.dim else 1
            spec.periodic[e] = int(self.periodic[e]) if e < self.dim else 0
        spec.level_min, spec.level_max = self.level_min, self.level_max
        n = len(self.leaves)
        keys = np.fromiter(itertools.chain.from_iterable(self.leaves), dtype=np.int32, count=4 * n)
        h = ctypes.c_void_p()
        rc = lib.g5_forest_create(ctypes.byref(spec), keys.ctypes.data_as(ctypes.c_void_p), n, ctypes.byref(h))
        if rc != 0:
            raise RuntimeError(f"g5_forest_create failed ({rc})")
        self._fcache = (h, self._leaves, n)
        return lib, h

    def _drop_forest(self) -> None:
        """Release the native forest (its leaves read out first when only it holds them)."""
        if self._fcache is None:
            return
        self.leaves  # noqa: B018
        from godunov_five_eq_gb300 import implem

        h, self._fcache = self._fcache[0], None
        implem.load_library().g5_forest_destroy(h)

    def __del__(self):
        try:
            if getattr(self, "_fcache", None) is not None:
                from godunov_five_eq_gb300 import implem

                implem.load_library().g5_forest_destroy(self._fcache[0])
                self._fcache = None
        except Exception:
            pass

    @staticmethod
    def _forest_leaves(lib, h) -> np.ndarray:
        import ctypes

        n = lib.g5_forest_num_leaves(h)
        out = np.empty((n, 4), np.int32)
        lib.g5_forest_leaves(h, out.ctypes.data_as(ctypes.c_void_p))
        return out

    def _leaves_changed(self, lib, h) -> None:
        """The native forest changed the leaves: they live there until read."""
        self._leaves = None
        self._fcache = (h, None, int(lib.g5_forest_num_leaves(h)))

    def balance(self) -> int:
        """Enforce 2:1 balance across faces, edges and corners (native forest)."""
        lib, h = self._forest()
        n = lib.g5_forest_balance(h)
        if n < 0:
            raise RuntimeError(f"g5_forest_balance failed ({n})")
        self._leaves_changed(lib, h)
        return int(n)

    # ------------------------------------------------------------ adaptation
    def adapt(self, flags) -> "RemapTable":
        """Apply per-block refine flags and return the old -> new block map.

        `flags` holds one ComputeRefineFlags code per owned block of the
        current table (ordered_leaves order): 2 refine, 0 coarsen, other
        values keep the block (scheme/ComputeRefineFlags.cpp:250-368).  The
        forest adaptation itself is p4est's (the reference's
        AMRManager::rebuild_from_context, SolverGodunovFiveEq.cpp:258-314);
        it runs in the native forest (g5_forest_adapt): refine every flagged
        block below level_max, restore 2:1 balance by refining, then coarsen
        each complete family of leaves above level_min whose 2^dim members
        are all flagged 0 and were not refined, unless the coarse block would
        touch a leaf two levels finer (such families are kept until none is
        left).  Every new block therefore comes from one old block (kept or
        refined once) or from the 2^dim old children of a family."""
        import ctypes

        flags = np.ascontiguousarray(np.asarray(flags).reshape(-1), np.int8)
        if flags.shape[0] != self._num_leaves():
            raise ValueError(f"expected {self._num_leaves()} flags, got {flags.shape[0]}")
        nc = 2**self.dim
        cap = max(1, flags.shape[0] * nc)
        kind = np.zeros(cap, np.int8)
        src = np.full((cap, nc), -1, np.int32)
        lib, h = self._forest()
        n_new = lib.g5_forest_adapt(
            h, flags.ctypes.data_as(ctypes.c_void_p), flags.shape[0], kind.ctypes.data_as(ctypes.c_void_p), src.ctypes.data_as(ctypes.c_void_p), cap
        )
        if n_new < 0:
            self._drop_forest()  # the forest may be half-adapted
            raise RuntimeError(f"g5_forest_adapt failed ({n_new})")
        self._leaves_changed(lib, h)
        return RemapTable(dim=self.dim, bsize=self.bsize, n_old=flags.shape[0], kind=kind[:n_new].copy(), src=src[:n_new].copy())

    # ------------------------------------------------------------------ tables
    def ordered_leaves(self):
        """Leaves in table order: brick tree (x fastest), then Morton order of
        the leaf origin at the finest level present (native forest)."""
        lib, h = self._forest()
        arr = self._forest_leaves(lib, h)
        return list(zip(*arr.T.tolist()))

    def build(self) -> BlockTable:
        """The block table of the current leaves (g5_forest_table): owned
        blocks in leaf order, their outside twins, the neighbour slots."""
        import ctypes

        lib, h = self._forest()
        n_owned, n_outside = ctypes.c_int32(), ctypes.c_int32()
        rc = lib.g5_forest_table_sizes(h, ctypes.byref(n_owned), ctypes.byref(n_outside))
        if rc != 0:
            raise RuntimeError(f"mesh not 2:1 balanced (g5_forest_table_sizes {rc})")
        no, nt = n_owned.value, n_outside.value
        ns, nc = 3**self.dim, 2**self.dim
        level = np.empty(no + nt, np.int32)
        coord = np.empty((no + nt, 3), np.int32)
        nbr = np.empty((no, ns, nc), np.int32)
        rel = np.empty((no, ns), np.int8)
        out_src = np.empty(nt, np.int32)
        out_normal = np.empty((nt, 3), np.int8)
        out_border = np.empty((nt, 6), np.int8)
        ptr = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
        rc = lib.g5_forest_table(h, ptr(level), ptr(coord), ptr(nbr), ptr(rel), ptr(out_src), ptr(out_normal), ptr(out_border))
        if rc != 0:
            raise RuntimeError(f"g5_forest_table failed ({rc})")
        return BlockTable(
            dim=self.dim,
            bsize=self.bsize,
            n_owned=no,
            n_outside=nt,
            level=level,
            coord=coord,
            nbr=nbr,
            nbr_rel=rel,
            out_src=out_src,
            out_normal=out_normal,
            out_border=out_border,
            inst=np.zeros(no + nt, dtype=np.int32),
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
