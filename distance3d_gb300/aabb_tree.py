"""AABB tree with distance3d's interface, backed by the GPU LBVH.

Mirrors distance3d aabb_tree.py: ``AabbTree`` (insert_aabbs, insert_aabb,
overlaps_aabb, overlaps_aabb_tree, get_root_aabb, external_data_list,
insert_index_list), ``all_aabbs_overlap`` and ``aabb_overlap``.

Leaf indices here are insertion order 0..n-1.  The reference numbers its
nodes differently (leaves interleave with branch nodes under incremental
insertion), and tells callers to translate indices through
``external_data_list`` / ``insert_index_list`` (aabb_tree.py:136-138,
176-178); both lists are kept consistent with these indices.  Pair sets are
identical to the reference's; the order of pairs is ascending instead of the
reference's depth-first order.  The tree is rebuilt on the GPU lazily, on the
first query after an insertion (the reference inserts incrementally,
aabb_tree.py:240-318).
"""
import numpy as np

from .bvh import LBVH

INDEX_NONE = -1


class AabbTree:
    """AABB tree for broad-phase collision detection (aabb_tree.py:15-191)."""

    def __init__(self, device="cuda"):
        self.device = device
        self.root = INDEX_NONE
        self.filled_len = 0
        self._boxes = []
        self.aabbs = np.empty((0, 3, 2))
        self.external_data_list = []
        self.insert_index_list = []
        self.insert_index_max = 0
        self._bvh = None

    def insert_aabbs(self, aabbs, external_data_list=None, pre_insertion_methode="none"):
        """Insert boxes (n,3,2).  ``pre_insertion_methode`` only changed the
        reference's incremental tree shape; the LBVH ignores it."""
        aabb_len = len(aabbs)
        if aabb_len == 0:
            return
        assert external_data_list is None or len(external_data_list) == aabb_len
        boxes = np.asarray(aabbs, dtype=np.float64).reshape(aabb_len, 3, 2)
        self.aabbs = np.concatenate([self.aabbs, boxes]) if self.filled_len else boxes.copy()
        self.filled_len += aabb_len
        self.external_data_list += list(external_data_list) if external_data_list is not None else [None] * aabb_len
        self.insert_index_list.extend(range(self.insert_index_max, self.insert_index_max + aabb_len))
        self.insert_index_max += aabb_len
        self.root = 0
        self._bvh = None

    def update_aabbs(self, aabbs):
        """Move every leaf to a new box (same count and order): the built
        tree is refit, not rebuilt (d3d_bvh_refit)."""
        boxes = np.asarray(aabbs, dtype=np.float64).reshape(-1, 3, 2)
        if len(boxes) != self.filled_len:
            raise ValueError(f"update_aabbs needs {self.filled_len} boxes, got {len(boxes)}")
        self.aabbs = boxes.copy()
        if self._bvh is not None and self.filled_len:
            self._bvh.refit(self.aabbs)

    def insert_aabb(self, aabb, external_data=None):
        self.insert_aabbs([aabb], [external_data])

    def _tree(self):
        if self._bvh is None:
            self._bvh = LBVH(self.aabbs, device=self.device)
        return self._bvh

    def overlaps_aabb(self, aabb):
        """(is_overlapping, leaf indices) for one query box (aabb_tree.py:161-181)."""
        if self.filled_len == 0:
            return False, np.array([], dtype=int)
        pairs = self._tree().query(np.asarray(aabb, dtype=np.float64).reshape(1, 3, 2)).cpu().numpy()
        overlaps = pairs[:, 0].astype(int)
        return len(overlaps) > 0, overlaps

    def overlaps_aabb_tree(self, other):
        """(is_overlapping, unique leaves of self, unique leaves of other,
        [(i_self, j_other), ...]) (aabb_tree.py:121-159)."""
        if self.filled_len == 0 or other.filled_len == 0:
            return False, np.array([], dtype=int), np.array([], dtype=int), []
        if other is self:
            p = self._tree().self_pairs().cpu().numpy().astype(int)
            n = self.filled_len
            diag = np.repeat(np.arange(n), 2).reshape(n, 2)
            diag = diag[np.all(self.aabbs[:, :, 0] <= self.aabbs[:, :, 1], axis=1)]
            pairs = np.concatenate([p, p[:, ::-1], diag])
            pairs = pairs[np.lexsort((pairs[:, 1], pairs[:, 0]))]
        else:
            pairs = self._tree().query(other.aabbs).cpu().numpy().astype(int)
        broad_pairs = [tuple(x) for x in pairs.tolist()]
        return (len(broad_pairs) > 0, np.unique(pairs[:, 0]) if len(pairs) else np.array([], dtype=int),
                np.unique(pairs[:, 1]) if len(pairs) else np.array([], dtype=int), broad_pairs)

    def get_root_aabb(self):
        """(3,2) box enclosing every leaf."""
        return np.stack([self.aabbs[:, :, 0].min(axis=0), self.aabbs[:, :, 1].max(axis=0)], axis=1)


def all_aabbs_overlap(aabbs1, aabbs2, device="cuda"):
    """Every overlapping (i, j), i in aabbs1, j in aabbs2 (aabb_tree.py:466-500):
    (unique i, unique j, [(i, j), ...]), computed on the GPU."""
    a1 = np.asarray(aabbs1, dtype=np.float64).reshape(-1, 3, 2)
    a2 = np.asarray(aabbs2, dtype=np.float64).reshape(-1, 3, 2)
    if len(a1) == 0 or len(a2) == 0:
        return np.array([], dtype=int), np.array([], dtype=int), []
    p = LBVH(a2, device=device).query(a1).cpu().numpy().astype(int)[:, ::-1]
    p = p[np.lexsort((p[:, 1], p[:, 0]))]
    return np.unique(p[:, 0]), np.unique(p[:, 1]), [tuple(x) for x in p.tolist()]


def aabb_overlap(aabb1, aabb2):
    """Closed-interval overlap of two (3,2) boxes (aabb_tree.py:504-527)."""
    a, b = np.asarray(aabb1), np.asarray(aabb2)
    return bool(a[0, 0] <= b[0, 1] and a[0, 1] >= b[0, 0] and a[1, 0] <= b[1, 1] and a[1, 1] >= b[1, 0]
                and a[2, 0] <= b[2, 1] and a[2, 1] >= b[2, 0])
