"""CPU restatement of bioshell-clustering's consumers of the crmsd matrix --
TEST INFRASTRUCTURE ONLY (the checker of the engine's clustering entry points).

Follows, step by step and with the same float32 arithmetic:
  * hierarchical_clustering      bioshell-clustering/src/hierarchical/hierarchical.rs:22-80
  * HierarchicalClusteringMatrix clustering_matrix.rs:11-74, including its quirks:
      - closest_elements scans j outer / i < j inner with a strict '<' from
        f32::MAX, so ties go to the first minimum in that order (:27-42);
      - update_distances passes sizes[j] as size_k for every k (:66);
      - replace_with_last swaps rows and copies one column but does not move
        `sizes` (:47-53);
  * merging rules                strategies/mod.rs:101-167
  * retrieve_clusters            hierarchical.rs:136-169
  * balance_clustering_tree      hierarchical.rs:86-99, if_rotate :242-291
  * medoid_by_min_max            hierarchical.rs:105-131
  * retrieve_outliers            hierarchical.rs:198-217
  * Optics                       bioshell-clustering/src/optics.rs:51-148, with
    neighbours as CartesianPoints::neighbors_of returns them (points_set.rs:150-169):
    the point itself included, d <= cutoff, stable sort by distance.
"""
from __future__ import annotations

import numpy as np

F32 = np.float32
F32_MAX = np.finfo(np.float32).max


# ------------------------------------------------------------------ rules
def single_link(si, sj, sk, dij, dik, djk):
    return F32(min(dik, djk))


def complete_link(si, sj, sk, dij, dik, djk):
    return F32(max(dik, djk))


def average_link(si, sj, sk, dij, dik, djk):
    d = F32(1.0) / F32(si + sj)
    return F32(d * F32(si) * dik + d * F32(sj) * djk)


def median_link(si, sj, sk, dij, dik, djk):
    return F32(F32(0.5) * dik + F32(0.5) * djk - F32(0.25) * dij)


def centroid_link(si, sj, sk, dij, dik, djk):
    d = F32(1.0) / F32(si + sj)
    return F32(d * F32(si) * dik + d * F32(sj) * djk - F32(si) * F32(sj) * d * d * dij)


def wards_method(si, sj, sk, dij, dik, djk):
    d = F32(1.0) / F32(si + sj + sk)
    return F32(d * F32(si + sk) * dik + d * F32(sj + sk) * djk - F32(sk) * d * dij)


RULES = {"single": single_link, "complete": complete_link, "average": average_link, "median": median_link,
         "centroid": centroid_link, "ward": wards_method}


class Node:
    __slots__ = ("id", "size", "dist", "left", "right")

    def __init__(self, id_, size, dist, left=None, right=None):
        self.id, self.size, self.dist, self.left, self.right = id_, size, F32(dist), left, right

    def is_leaf(self):
        return self.left is None and self.right is None


def hierarchical_clustering(n, dist, rule):
    m = [[F32(0.0)] * n for _ in range(n)]
    for i in range(1, n):
        for j in range(i):
            v = F32(dist(i, j))
            m[i][j] = v
            m[j][i] = v
    sizes = [1] * n
    order = n
    clusters = {i: Node(i, 1, 0.0) for i in range(n)}
    cur = n
    while len(clusters) > 1:
        mn, mi, mj = F32_MAX, 0, 0
        for j in range(1, order):
            for i in range(j):
                if m[i][j] < mn:
                    mn, mi, mj = m[i][j], i, j
        i, j = mi, mj
        ci, cj = clusters.pop(i), clusters.pop(j)
        c = Node(cur, ci.size + cj.size, m[i][j], ci, cj)
        clusters[i] = c
        # update_distances(i, j, rule, new_index = i)
        size_i, size_j = sizes[i], sizes[j]
        res = [rule(size_i, size_j, sizes[j], m[i][j], m[i][k], m[j][k]) for k in range(order)]
        for k in range(order):
            m[i][k] = res[k]
            m[k][i] = res[k]
        m[i][i] = F32(0.0)
        sizes[i] = size_j + size_i
        last = order - 1
        if j < last:
            clusters[j] = clusters.pop(last)
            # replace_with_last(j)
            order -= 1
            m[j], m[order] = m[order], m[j]
            for r in range(order):
                m[r][j] = m[r][order]
        else:
            order -= 1
        cur += 1
    return clusters[0]


def preorder_leaves(node):
    out, stack = [], [node]
    while stack:
        nd = stack.pop()
        if nd.is_leaf():
            out.append(nd.id)
        else:
            if nd.right is not None:
                stack.append(nd.right)
            if nd.left is not None:
                stack.append(nd.left)
    return out


def retrieve_clusters(root, max_distance):
    """The reference's recursion (hierarchical.rs:136-169) with an explicit
    stack, so that deep trees (single linkage of thousands of items) do not
    hit Python's recursion limit; clusters come out in the same order."""
    max_distance = F32(max_distance)
    out = []
    if root.dist <= max_distance:
        out.append(root)
        return out
    stack = [(False, root)]  # (emit, node): emit a cluster, or recurse into a node
    while stack:
        emit, node = stack.pop()
        if emit:
            out.append(node)
        elif node.is_leaf():
            out.append(node)
        elif node.dist > max_distance:
            for ch in (node.right, node.left):  # pushed in reverse: left is handled first
                if ch is not None:
                    stack.append((ch.dist <= max_distance, ch))
    return out


def _rotate(node):
    if node.left is not None:
        _rotate(node.left)
    if node.right is not None:
        _rotate(node.right)
    node.left, node.right = node.right, node.left


def _leftmost(c):
    while c.left is not None:
        c = c.left
    return c.id


def _rightmost(c):
    while c.right is not None:
        c = c.right
    return c.id


def _if_rotate(c, dist):
    if c.is_leaf():
        return False, False
    left, right = c.left, c.right
    if right.is_leaf() and left.is_leaf():
        return False, False
    if right.is_leaf():
        if dist(right.id, _leftmost(left)) < dist(right.id, _rightmost(left)):
            return True, False
        return False, False
    if left.is_leaf():
        if dist(left.id, _leftmost(right)) > dist(left.id, _rightmost(right)):
            return False, True
        return False, False
    rr, rl, lr, ll = _rightmost(right), _leftmost(right), _rightmost(left), _leftmost(left)
    d = [dist(lr, rl), dist(ll, rl), dist(lr, rr), dist(ll, rr)]
    k = min(range(4), key=lambda t: (d[t], t))
    return {1: (True, False), 2: (False, True), 3: (True, True)}.get(k, (False, False))


def balance_clustering_tree(root, dist):
    def rec(node):
        if node.left is not None:
            rec(node.left)
        if node.right is not None:
            rec(node.right)
        rl, rr = _if_rotate(node, dist)
        if rl:
            _rotate(node.left)
        if rr:
            _rotate(node.right)

    rec(root)


def medoid_by_min_max(cluster, dist):
    members = preorder_leaves(cluster)
    if len(members) == 1:
        return members[0]
    best, bi = F32_MAX, 0
    for i in range(len(members)):
        mx = -F32_MAX
        for j in range(len(members)):
            if i != j:
                d = F32(dist(members[i], members[j]))
                if d > mx:
                    mx = d
        if mx < best:
            best, bi = mx, i
    return members[bi]


def retrieve_outliers(n, dist, cutoff):
    out = []
    if n < 2:
        return out
    for i in range(n):
        mn = F32_MAX
        for j in range(n):
            if i != j:
                d = F32(dist(i, j))
                if d < mn:
                    mn = d
        if mn > F32(cutoff):
            out.append(i)
    return out


# ------------------------------------------------------------------ OPTICS
def optics(n, dist, eps, min_points):
    """Returns (clustering_order, reachability, clusters) as the reference's
    Optics does; distances are f64."""
    undefined = eps * 10.0
    reach = [undefined] * n
    processed = [False] * n
    order = []

    def neighbors_of(i):
        nb = [(j, float(dist(i, j))) for j in range(n)]
        nb = [(j, d) for (j, d) in nb if d <= eps]
        nb.sort(key=lambda t: t[1])
        return nb

    def update(nb, seeds):
        core = nb[min_points - 1][1]
        for (j, d) in nb:
            if processed[j]:
                continue
            new = max(d, core)
            if reach[j] == undefined:
                seeds.append(j)
            if reach[j] > new:
                reach[j] = new
        seeds.sort(key=lambda t: reach[t])

    for i in range(n):
        if processed[i]:
            continue
        order.append(i)
        nb = neighbors_of(i)
        processed[i] = True
        if len(nb) < min_points:
            continue
        seeds = []
        update(nb, seeds)
        while seeds:
            pi = seeds[0]
            seeds[0] = seeds[-1]
            seeds.pop()
            seeds.sort(key=lambda t: reach[t])
            order.append(pi)
            nbs = neighbors_of(pi)
            processed[pi] = True
            if len(nbs) < min_points:
                continue
            update(nbs, seeds)
    clusters = []
    start = 0
    for k in range(1, n):
        if reach[order[k]] == undefined:
            clusters.append(order[start:k])
            start = k
    clusters.append(order[start:n])
    return order, reach, clusters


# ------------------------------------------- vectorised hierarchical runs
# The same steps as hierarchical_clustering above (hierarchical.rs:22-80 with
# clustering_matrix.rs:27-74), one merge at a time with numpy over a float32
# square matrix, so that the 500-structure workload clusters in about a
# second per rule.  Each rule evaluates in the reference's operation order,
# one float32 rounding per operation (numpy does not contract a * b + c).
def _rule_rows(rule, si, sj, sk, dij, dik, djk):
    if rule == "single":
        return np.minimum(dik, djk)
    if rule == "complete":
        return np.maximum(dik, djk)
    if rule == "average":
        d = F32(1.0) / F32(si + sj)
        return (d * F32(si)) * dik + (d * F32(sj)) * djk
    if rule == "median":
        return (F32(0.5) * dik + F32(0.5) * djk) - F32(0.25) * dij
    if rule == "centroid":
        d = F32(1.0) / F32(si + sj)
        return ((d * F32(si)) * dik + (d * F32(sj)) * djk) - (((F32(si) * F32(sj)) * d) * d) * dij
    if rule == "ward":
        d = F32(1.0) / F32(si + sj + sk)
        return ((d * F32(si + sk)) * dik + (d * F32(sj + sk)) * djk) - (F32(sk) * d) * dij
    raise ValueError(rule)


class HierRun:
    """One hierarchical_clustering run over a square matrix, advanced merge by
    merge.  ``merges`` rows are (left id, right id, new id, size) -- leaves
    are 0..n-1, the s-th merge creates node n + s -- and ``dist`` holds the
    float32 merging distances."""

    def __init__(self, sq, rule):
        m = np.array(sq, dtype=F32, copy=True)
        n = m.shape[0]
        np.fill_diagonal(m, F32(0.0))
        self.m, self.n, self.rule = m, n, rule
        self.sizes = [1] * n           # clustering_matrix.rs sizes (not moved by replace_with_last)
        self.ids = list(range(n))      # node id at each matrix position
        self.node_size = {i: 1 for i in range(n)}
        self.order, self.cur = n, n
        self.merges, self.dist = [], []
        self._upper = np.triu(np.ones((n, n), dtype=bool), 1)

    def done(self):
        return self.order <= 1

    def closest(self):
        """(i, j, minimum, second smallest candidate): the first minimum of the
        j-outer, i-inner scan over i < j (clustering_matrix.rs:27-42)."""
        o = self.order
        u = np.where(self._upper[:o, :o], self.m[:o, :o], np.inf).T.ravel()
        k = int(np.argmin(u))
        mn = u[k]
        if not mn < F32_MAX:
            return 0, 0, F32_MAX, np.inf
        j, i = divmod(k, o)
        second = np.partition(u, 1)[1] if u.size > 1 else np.inf
        return i, j, mn, second

    def merge(self, i, j):
        m, o = self.m, self.order
        dij = m[i, j]
        left, right = self.ids[i], self.ids[j]
        size = self.node_size[left] + self.node_size[right]
        self.merges.append((left, right, self.cur, size))
        self.dist.append(F32(dij))
        self.node_size[self.cur] = size
        self.ids[i] = self.cur
        si, sj = self.sizes[i], self.sizes[j]
        res = _rule_rows(self.rule, si, sj, self.sizes[j], dij, m[i, :o].copy(), m[j, :o].copy()).astype(F32)
        m[i, :o] = res
        m[:o, i] = res
        m[i, i] = F32(0.0)
        self.sizes[i] = sj + si
        last = o - 1
        if j < last:
            self.ids[j] = self.ids[last]
            self.order = o - 1
            o = self.order
            m[[j, o]] = m[[o, j]]
            m[:o, j] = m[:o, o]
        else:
            self.order = o - 1
        self.cur += 1

    def run(self):
        while not self.done():
            i, j, _, _ = self.closest()
            self.merge(i, j)
        return self.result()

    def result(self):
        n = self.n
        merges = np.array(self.merges, dtype=np.int64).reshape(max(n - 1, 0), 4)
        return merges, np.array(self.dist, dtype=F32)


def hierarchical_merges(sq, rule):
    """merges and merging distances of hierarchical_clustering(sq, rule)."""
    return HierRun(sq, rule).run()


def tree_from_merges(n, merges, dist):
    """The Node tree of a merge list (root: the last merge)."""
    nodes = {i: Node(i, 1, 0.0) for i in range(n)}
    for (a, b, c, s), d in zip(merges, dist):
        nodes[int(c)] = Node(int(c), int(s), d, nodes[int(a)], nodes[int(b)])
    return nodes[2 * n - 2] if n > 1 else nodes.get(0)


def cut_labels(n, merges, dist, cutoff):
    """Cluster index per item: the k-th cluster retrieve_clusters returns
    (hierarchical.rs:136-169) is label k."""
    labels = np.zeros(n, dtype=np.int64)
    if n == 0:
        return labels
    root = tree_from_merges(n, merges, dist)
    for k, c in enumerate(retrieve_clusters(root, cutoff)):
        labels[preorder_leaves(c)] = k
    return labels


def lockstep(sq_a, sq_b, rule):
    """Runs the clustering of two nearby matrices side by side.  While both
    runs take the same merges, it records per merge the largest difference
    between their working matrices (delta) and the slack of run b's merge:
    the least, over every other candidate c, of b[c] - b[min] - |a[c] - b[c]|
    - |a[min] - b[min]|.  A merge with slack > 0 is taken by run a as well,
    whatever the two matrices' differences do to the scan; slack <= 0 marks
    a merge that could go the other way.  Returns both runs' (merges, dist),
    the index of the first merge where they part (None if never), and the
    per-merge delta and slack up to that merge."""
    a, b = HierRun(sq_a, rule), HierRun(sq_b, rule)
    delta, slack, split = [], [], None
    while not b.done():
        o = b.order
        up = b._upper[:o, :o]
        bm = b.m[:o, :o].astype(np.float64)
        d = np.abs(a.m[:o, :o].astype(np.float64) - bm)
        delta.append(float(d[up].max()) if o > 1 else 0.0)
        ia, ja, _, _ = a.closest()
        ib, jb, mn, _ = b.closest()
        if o > 2:
            margin = np.where(up, bm - float(mn) - d, np.inf)
            margin[ib, jb] = np.inf
            slack.append(float(margin.min()) - float(d[ib, jb]))
        else:
            slack.append(np.inf)
        if (ia, ja) != (ib, jb):
            split = len(delta) - 1
            break
        a.merge(ia, ja)
        b.merge(ib, jb)
    return a.run(), b.run(), split, np.array(delta), np.array(slack)
