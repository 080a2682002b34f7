"""Clustering of a crmsd matrix through the engine's C ABI (host code in
``csrc/cluster.cpp``), mirroring bioshell-clustering's consumers:

* ``hierarchical_clustering(matrix, rule)``  -- hierarchical.rs:22-80
* ``cut_tree(tree, cutoff)``                   -- labels of retrieve_clusters, hierarchical.rs:136-169
* ``optics(matrix, eps, min_points)``          -- optics.rs:51-148
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from . import lib as _l
from .crmsd import CrmsdMatrix


@dataclass
class ClusteringTree:
    """n-1 merges: merges[s] = (left id, right id, new id, size), dist[s]."""

    n: int
    merges: np.ndarray
    dist: np.ndarray

    def leaves_preorder(self):
        """Leaf ids in depth-first preorder (the order retrieve_data returns)."""
        if self.n == 0:
            return []
        kids = {int(m[2]): (int(m[0]), int(m[1])) for m in self.merges}
        out, stack = [], [2 * self.n - 2 if self.n > 1 else 0]
        while stack:
            v = stack.pop()
            if v < self.n:
                out.append(v)
            else:
                a, b = kids[v]
                stack.append(b)
                stack.append(a)
        return out


def _tri(matrix: CrmsdMatrix):
    if matrix.layout != "triangle":
        raise ValueError("clustering takes the packed-triangle layout")
    v = np.ascontiguousarray(matrix.values)
    if v.dtype == np.float64:
        return v, _l.OUT_TYPE["f64"]
    if v.dtype == np.float32:
        return v, _l.OUT_TYPE["f32"]
    raise TypeError("matrix values must be float64 or float32")


def _check(st, what):
    if st != _l.BS_OK:
        raise _l.CrmsdError(st, what)


def hierarchical_clustering(matrix: CrmsdMatrix, rule: str = "single", engine=None) -> ClusteringTree:
    """Agglomerative clustering of the matrix; on the GPU of ``engine`` when
    one is given (same merges, bit for bit), else on the host."""
    v, ot = _tri(matrix)
    n = matrix.n
    merges = np.zeros((max(n - 1, 0), 4), dtype=np.int64)
    dist = np.zeros(max(n - 1, 0), dtype=np.float32)
    mp = merges.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))
    dp = dist.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
    if engine is not None:
        engine._check(_l.load().bs_hierarchical_gpu(engine._h, v.ctypes.data, n, ot, _l.LINK[rule], mp, dp))
    else:
        _check(_l.load().bs_hierarchical(v.ctypes.data, n, ot, _l.LINK[rule], mp, dp), "bs_hierarchical")
    return ClusteringTree(n, merges, dist)


def cut_tree(tree: ClusteringTree, cutoff: float) -> np.ndarray:
    labels = np.zeros(tree.n, dtype=np.int64)
    st = _l.load().bs_cut_tree(tree.merges.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                               tree.dist.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), tree.n, float(cutoff),
                               labels.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)))
    _check(st, "bs_cut_tree")
    return labels


def optics(matrix: CrmsdMatrix, eps: float, min_points: int):
    """(clustering order, reachability in that order, cluster index per item)."""
    v, ot = _tri(matrix)
    n = matrix.n
    order = np.zeros(n, dtype=np.int64)
    reach = np.zeros(n, dtype=np.float64)
    cl = np.zeros(n, dtype=np.int64)
    st = _l.load().bs_optics(v.ctypes.data, n, ot, float(eps), int(min_points),
                             order.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                             reach.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                             cl.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)))
    _check(st, "bs_optics")
    return order, reach, cl


def optics_neighbors(row_ptr, col, dist, eps: float, min_points: int):
    """OPTICS over sparse neighbour lists (CSR, as ``Engine.neighbors`` returns
    them): (clustering order, reachability in that order, cluster index per
    item) -- the same as ``optics`` on a dense f32 matrix holding the values."""
    row_ptr = np.ascontiguousarray(row_ptr, dtype=np.int64)
    col = np.ascontiguousarray(col, dtype=np.int32)
    dist = np.ascontiguousarray(dist, dtype=np.float32)
    n = row_ptr.shape[0] - 1
    order = np.zeros(n, dtype=np.int64)
    reach = np.zeros(n, dtype=np.float64)
    cl = np.zeros(n, dtype=np.int64)
    st = _l.load().bs_optics_neighbors(row_ptr.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                                       col.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                                       dist.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), n, float(eps),
                                       int(min_points), order.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                                       reach.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                       cl.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)))
    _check(st, "bs_optics_neighbors")
    return order, reach, cl


def neighbors_from_dense(m, eps: float):
    """CSR neighbour lists of a dense symmetric matrix: for every row i the
    columns j != i with m[i, j] <= eps, ordered by (distance, j)."""
    m = np.asarray(m, dtype=np.float32)
    n = m.shape[0]
    rows, cols, vals = [], [], []
    row_ptr = np.zeros(n + 1, dtype=np.int64)
    for i in range(n):
        j = np.flatnonzero(m[i] <= eps)
        j = j[j != i]
        o = np.lexsort((j, m[i, j]))
        cols.append(j[o].astype(np.int32))
        vals.append(m[i, j[o]])
        row_ptr[i + 1] = row_ptr[i] + len(j)
    col = np.concatenate(cols) if cols else np.zeros(0, np.int32)
    val = np.concatenate(vals) if vals else np.zeros(0, np.float32)
    return row_ptr, col, val
