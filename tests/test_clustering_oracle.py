"""Pins the clustering restatement (oracle/clustering.py) on the reference's
own hierarchical-clustering tests, replayed from their recorded inputs and
expected outputs (bioshell-clustering/tests/test_hierarchical.rs:10-71)."""
import json
import os

import numpy as np
import pytest

from oracle import clustering as C

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "hierarchical_reference_tests.json")


def _ref():
    with open(GOLDEN) as fh:
        return json.load(fh)


def test_cluster_numbers():
    t = _ref()["cluster_numbers"]
    data = np.array(t["data"], dtype=np.float32)
    dist = lambda a, b: np.float32(abs(data[a] - data[b]))  # noqa: E731
    root = C.hierarchical_clustering(len(data), dist, C.single_link)
    assert root.size == 4
    assert [float(data[i]) for i in C.preorder_leaves(root)] == [float(np.float32(v)) for v in t["order"]]
    C.balance_clustering_tree(root, dist)
    assert [float(data[i]) for i in C.preorder_leaves(root)] == [float(np.float32(v)) for v in t["order_balanced"]]


def test_cluster_letters():
    t = _ref()["cluster_letters"]
    data = t["data"]
    dist = lambda a, b: np.float32(abs(ord(data[a]) - ord(data[b])))  # noqa: E731
    root = C.hierarchical_clustering(len(data), dist, C.single_link)
    assert root.size == len(data)
    assert [data[i] for i in C.preorder_leaves(root)] == t["order"]
    C.balance_clustering_tree(root, dist)
    assert [data[i] for i in C.preorder_leaves(root)] == t["order_balanced"]


def test_cluster_distance_matrix():
    t = _ref()["cluster_distance_matrix"]
    labels = []
    for a, b, _ in t["tsv"]:
        for x in (a, b):
            if x not in labels:
                labels.append(x)
    n = len(labels)
    m = np.zeros((n, n), dtype=np.float32)
    for a, b, v in t["tsv"]:
        i, j = labels.index(a), labels.index(b)
        m[i, j] = m[j, i] = v
    dist = lambda i, j: np.float32(0.0) if i == j else m[i, j]  # noqa: E731
    root = C.hierarchical_clustering(n, dist, C.single_link)
    clusters = sorted(C.retrieve_clusters(root, t["cutoff"]), key=lambda c: c.size)
    assert len(clusters) == t["n_clusters"]
    assert sum(c.size for c in clusters) == t["n_points"]
    assert clusters[-1].size == t["largest"]
    for c in clusters[:3]:
        assert C.medoid_by_min_max(c, dist) == C.preorder_leaves(c)[0]


def test_all_rules_run_and_merge_everything():
    rng = np.random.default_rng(0)
    pts = rng.normal(size=(30, 2)).astype(np.float32)
    dist = lambda i, j: np.float32(np.linalg.norm(pts[i] - pts[j]))  # noqa: E731
    for name, rule in C.RULES.items():
        root = C.hierarchical_clustering(30, dist, rule)
        assert root.size == 30 and sorted(C.preorder_leaves(root)) == list(range(30)), name


def test_optics_two_blobs():
    rng = np.random.default_rng(1)
    a = rng.normal(size=(20, 2)) * 0.3
    b = rng.normal(size=(20, 2)) * 0.3 + 3.0
    pts = np.concatenate([a, b])
    dist = lambda i, j: float(np.sum((pts[i] - pts[j]) ** 2))  # noqa: E731  (squared, as the reference test)
    order, reach, clusters = C.optics(40, dist, 0.5, 5)
    assert sorted(order) == list(range(40))
    sizes = sorted(len(c) for c in clusters)
    assert sizes[-2:] == [20, 20]


@pytest.mark.parametrize("rule", list(C.RULES))
@pytest.mark.parametrize("seed,ties", [(0, False), (1, True)])
def test_vectorised_runs_equal_the_loop_restatement(rule, seed, ties):
    """HierRun (numpy, one merge at a time) takes the same merges with the same
    float32 distances as the loop restatement of hierarchical.rs."""
    rng = np.random.default_rng(seed)
    n = 40
    if ties:
        sq = rng.integers(1, 6, size=(n, n)).astype(np.float64)
    else:
        pts = rng.normal(size=(n, 3))
        sq = np.linalg.norm(pts[:, None] - pts[None], axis=2)
    sq = np.triu(sq, 1)
    sq = sq + sq.T
    dist = lambda i, j: np.float32(0.0) if i == j else np.float32(sq[i, j])  # noqa: E731
    root = C.hierarchical_clustering(n, dist, C.RULES[rule])
    merges, d = C.hierarchical_merges(sq.astype(np.float32), rule)

    def walk(nd, out):
        if not nd.is_leaf():
            walk(nd.left, out)
            walk(nd.right, out)
            out.append((nd.id, nd.left.id, nd.right.id, nd.size, float(nd.dist)))
        return out

    assert sorted(walk(root, [])) == sorted(walk(C.tree_from_merges(n, merges, d), []))
    for cut in (1.5, 2.5, float(np.median(d))):
        want = np.zeros(n, dtype=np.int64)
        for k, c in enumerate(C.retrieve_clusters(root, cut)):
            want[C.preorder_leaves(c)] = k
        np.testing.assert_array_equal(C.cut_labels(n, merges, d, cut), want)


def test_lockstep_reports_where_runs_part():
    """Two matrices that differ in one entry part exactly where that entry
    decides a merge, and the slack recorded there is not positive."""
    rng = np.random.default_rng(4)
    pts = rng.normal(size=(30, 3))
    sq = np.linalg.norm(pts[:, None] - pts[None], axis=2).astype(np.float32)
    (ma, da), (mb, db), split, delta, slack = C.lockstep(sq, sq, "average")
    assert split is None and np.all(delta == 0.0) and np.all(slack >= 0.0)
    np.testing.assert_array_equal(ma, mb)
    iu = np.triu_indices(30, 1)
    k = int(np.argsort(sq[iu])[1])  # the second closest pair becomes the closest
    i, j = iu[0][k], iu[1][k]
    sq2 = sq.copy()
    sq2[i, j] = sq2[j, i] = np.float32(sq[iu].min() - 1e-3)
    _, _, split, delta, slack = C.lockstep(sq2, sq, "average")
    assert split == 0 and slack[0] <= 0.0 and delta[0] > 0.0
