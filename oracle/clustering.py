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
    max_distance = F32(max_distance)
    out = []

    def rec(node):
        if node.is_leaf():
            out.append(node)
        elif node.dist > max_distance:
            for ch in (node.left, node.right):
                if ch is not None:
                    if ch.dist <= max_distance:
                        out.append(ch)
                    else:
                        rec(ch)

    if root.dist <= max_distance:
        out.append(root)
    else:
        rec(root)
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
