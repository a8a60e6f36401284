"""Python restatement of the block-forest algorithms (balance, adaptation
with the old -> new block map, leaf order, block table).

Test infrastructure, like the rest of oracle/: it checks the native forest of
libg5gpu.so (godunov_five_eq_gb300/csrc/g5_forest.cpp) on random meshes (both
must give the same leaves, remap tables and block tables), and it builds the
meshes of bench.py's CPU reference arm, which then loads no library of the
product.  PyBlockMesh never touches the native forest: every BlockMesh
operation that would call it is overridden here."""
import itertools

import numpy as np

from godunov_five_eq_gb300.mesh import REMAP_COARSENED, REMAP_REFINED, BlockMesh, BlockTable, RemapTable, _morton


class PyBlockMesh(BlockMesh):
    """BlockMesh with the pure-Python balance / adapt / order / build."""

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
