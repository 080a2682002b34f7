"""Hierarchical clustering on the GPU (bs_hierarchical_gpu): the same merges
and merge distances as the oracle's restatement of hierarchical.rs
(oracle.clustering, itself pinned on the reference's test vectors), bit for
bit, for every merge rule -- with exact ties, f32 and f64 inputs -- and the
same as the host version."""
import numpy as np
import pytest

from bioshell_gb300 import clustering as K
from bioshell_gb300 import synth
from bioshell_gb300.crmsd import CrmsdMatrix
from oracle import clustering as C

pytestmark = pytest.mark.gpu

RULES = ["single", "complete", "average", "median", "centroid", "ward"]


def _tri(sq, dtype):
    n = sq.shape[0]
    iu = np.triu_indices(n, 1)
    return CrmsdMatrix(n, np.ascontiguousarray(sq[iu], dtype=dtype), "triangle")


@pytest.mark.parametrize("rule", RULES)
@pytest.mark.parametrize("ties", [False, True])
def test_gpu_merges_equal_host(engine, rule, ties):
    rng = np.random.default_rng(7 + RULES.index(rule))
    pts = rng.normal(size=(257, 3)) * 4.0
    if ties:
        pts = np.round(pts)  # many equal distances
    sq = np.linalg.norm(pts[:, None] - pts[None], axis=2)
    # the matrix the reference fills: every distance rounded to f32
    want_merges, want_dist = C.hierarchical_merges(sq.astype(np.float32), rule)
    for dtype in (np.float32, np.float64):
        m = _tri(sq, dtype)
        dev = K.hierarchical_clustering(m, rule, engine=engine)
        np.testing.assert_array_equal(dev.merges, want_merges)
        np.testing.assert_array_equal(dev.dist, want_dist)
        host = K.hierarchical_clustering(m, rule)
        np.testing.assert_array_equal(dev.merges, host.merges)
        np.testing.assert_array_equal(dev.dist, host.dist)


def test_gpu_crmsd_matrix(engine):
    rng = np.random.default_rng(21)
    x = synth.decoys(synth.base_chain(80, rng), 1800, rng, sigma=(0.3, 4.0))
    m = engine.all_vs_all(x)
    n = x.shape[0]
    sq = np.zeros((n, n))
    sq[np.triu_indices(n, 1)] = m.values
    sq = (sq + sq.T).astype(np.float32)
    for rule in ("single", "average", "ward"):
        want_merges, want_dist = C.hierarchical_merges(sq, rule)
        dev = K.hierarchical_clustering(m, rule, engine=engine)
        np.testing.assert_array_equal(dev.merges, want_merges)
        np.testing.assert_array_equal(dev.dist, want_dist)
        host = K.hierarchical_clustering(m, rule)
        np.testing.assert_array_equal(dev.merges, host.merges)
        np.testing.assert_array_equal(K.cut_tree(dev, 2.0), C.cut_labels(n, want_merges, want_dist, 2.0))


def test_gpu_small(engine):
    for n in (0, 1, 2, 3):
        m = _tri(np.ones((n, n)) - np.eye(n), np.float32)
        host = K.hierarchical_clustering(m, "single")
        dev = K.hierarchical_clustering(m, "single", engine=engine)
        np.testing.assert_array_equal(dev.merges, host.merges)
