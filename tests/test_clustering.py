"""The engine's clustering of a crmsd matrix (host code behind the C ABI)
against the oracle's restatement of bioshell-clustering, bit for bit:
same merges, same f32 merging distances, same labels, same OPTICS order."""
import json
import os

import numpy as np
import pytest

from bioshell_gb300 import clustering as K
from bioshell_gb300.crmsd import CrmsdMatrix
from oracle import clustering as C

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "hierarchical_reference_tests.json")


def _matrix(sq, dtype=np.float64):
    n = sq.shape[0]
    iu = np.triu_indices(n, 1)
    return CrmsdMatrix(n, np.ascontiguousarray(sq[iu], dtype=dtype), "triangle")


def _oracle_merges(root):
    out = []

    def rec(nd):
        if nd.is_leaf():
            return
        rec(nd.left)
        rec(nd.right)
        out.append((nd.id, nd.left.id, nd.right.id, nd.size, float(nd.dist)))

    rec(root)
    return sorted(out)


@pytest.mark.parametrize("rule", list(C.RULES))
@pytest.mark.parametrize("seed,ties", [(0, False), (1, True), (2, True)])
def test_hierarchical_matches_oracle(enginelib, rule, seed, ties):
    rng = np.random.default_rng(seed)
    n = 60
    if ties:  # integer distances force many equal minima (tie-breaking order)
        sq = rng.integers(1, 6, size=(n, n)).astype(np.float64)
    else:
        pts = rng.normal(size=(n, 3))
        sq = np.linalg.norm(pts[:, None] - pts[None], axis=2)
    sq = np.triu(sq, 1)
    sq = sq + sq.T
    m = _matrix(sq)
    tree = K.hierarchical_clustering(m, rule)
    dist = lambda i, j: np.float32(0.0) if i == j else np.float32(sq[i, j])  # noqa: E731
    root = C.hierarchical_clustering(n, dist, C.RULES[rule])
    got = sorted((int(a[2]), int(a[0]), int(a[1]), int(a[3]), float(d)) for a, d in zip(tree.merges, tree.dist))
    assert got == _oracle_merges(root)
    assert tree.leaves_preorder() == C.preorder_leaves(root)
    for cut in (0.5, 1.5, 2.5, float(np.median(tree.dist))):
        labels = K.cut_tree(tree, cut)
        ref = C.retrieve_clusters(root, cut)
        want = np.zeros(n, dtype=np.int64)
        for k, c in enumerate(ref):
            want[C.preorder_leaves(c)] = k
        np.testing.assert_array_equal(labels, want)


def test_reference_vectors_through_engine(enginelib):
    t = json.load(open(GOLDEN))
    data = np.array(t["cluster_numbers"]["data"], dtype=np.float32)
    sq = np.abs(data[:, None] - data[None]).astype(np.float64)
    tree = K.hierarchical_clustering(_matrix(sq, np.float32), "single")
    assert [float(data[i]) for i in tree.leaves_preorder()] == [float(np.float32(v)) for v in t["cluster_numbers"]["order"]]
    letters = t["cluster_letters"]["data"]
    codes = np.array([ord(c) for c in letters], dtype=np.float64)
    tree = K.hierarchical_clustering(_matrix(np.abs(codes[:, None] - codes[None])), "single")
    assert [letters[i] for i in tree.leaves_preorder()] == t["cluster_letters"]["order"]
    d5 = t["cluster_distance_matrix"]
    labels = []
    for a, b, _ in d5["tsv"]:
        for x in (a, b):
            if x not in labels:
                labels.append(x)
    sq = np.zeros((len(labels), len(labels)))
    for a, b, v in d5["tsv"]:
        sq[labels.index(a), labels.index(b)] = sq[labels.index(b), labels.index(a)] = v
    tree = K.hierarchical_clustering(_matrix(sq, np.float32), "single")
    lab = K.cut_tree(tree, d5["cutoff"])
    sizes = sorted(np.bincount(lab))
    assert len(sizes) == d5["n_clusters"] and sizes[-1] == d5["largest"] and sum(sizes) == d5["n_points"]


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_optics_matches_oracle(enginelib, seed):
    rng = np.random.default_rng(seed)
    pts = np.concatenate([rng.normal(size=(25, 2)) * 0.4, rng.normal(size=(25, 2)) * 0.4 + 3.0,
                          rng.uniform(-3, 6, size=(10, 2))])
    sq = np.linalg.norm(pts[:, None] - pts[None], axis=2)
    m = _matrix(sq)
    for eps, mp in ((0.8, 4), (1.2, 6), (0.3, 2)):
        order, reach, cl = K.optics(m, eps, mp)
        o2, r2, c2 = C.optics(60, lambda i, j: sq[i, j], eps, mp)
        assert list(order) == o2
        np.testing.assert_array_equal(reach, np.array([r2[k] for k in o2]))
        want = np.zeros(60, dtype=np.int64)
        for k, c in enumerate(c2):
            want[c] = k
        np.testing.assert_array_equal(cl, want)


@pytest.mark.parametrize("seed", [0, 3])
def test_optics_on_neighbor_lists_equals_dense(enginelib, seed):
    """OPTICS over sparse (CSR) neighbour lists gives the dense f32 matrix's
    order, reachability and labels -- including exact ties and zero distances
    (identical items), where the point itself must sit in its stable-sort
    place."""
    rng = np.random.default_rng(seed)
    pts = np.concatenate([rng.normal(size=(30, 2)) * 0.4, rng.normal(size=(30, 2)) * 0.4 + 3.0,
                          rng.uniform(-3, 6, size=(10, 2))])
    pts = np.round(pts, 1)          # ties
    pts[5] = pts[4]                 # identical items: distance 0
    pts[40] = pts[41] = pts[45]
    sq = np.linalg.norm(pts[:, None] - pts[None], axis=2).astype(np.float32)
    m = _matrix(sq, np.float32)
    for eps, mp in ((0.8, 4), (1.2, 6), (0.3, 2), (0.5, 1)):
        rp, col, val = K.neighbors_from_dense(sq, eps)
        o1, r1, c1 = K.optics(m, eps, mp)
        o2, r2, c2 = K.optics_neighbors(rp, col, val, eps, mp)
        np.testing.assert_array_equal(o1, o2)
        np.testing.assert_array_equal(r1, r2)
        np.testing.assert_array_equal(c1, c2)


def test_degenerate_sizes(enginelib):
    for n in (0, 1, 2):
        m = CrmsdMatrix(n, np.ones(n * (n - 1) // 2), "triangle")
        tree = K.hierarchical_clustering(m, "average")
        assert tree.merges.shape == (max(n - 1, 0), 4)
        assert len(K.cut_tree(tree, 0.5)) == n
