"""Cluster labels from the engine's crmsd matrix against cluster labels from the
FP64 oracle's matrix, on the 500-decoy workload (500 decoys of a 64-residue
chain, 124,750 pairs): what a user of bioshell-clustering sees when the
matrix comes from the engine instead of an FP64 crmsd.

The claim tested: labels are identical wherever no decision of the clustering
lies within the engine's distance error of a threshold.  Each (rule, cutoff)
or (eps, min_points) instance is classified before its labels are compared:

* hierarchical (hierarchical.rs:22-80, clustering_matrix.rs:27-42): the two
  matrices are clustered side by side (oracle.clustering.lockstep).  At each
  merge the oracle run's choice, the minimum, is compared with every other
  candidate c: when b[c] - b[min] is within the two runs' differences at c
  and at the minimum (|a[c] - b[c]| + |a[min] - b[min]|), the merge could
  go the other way, and the rule's run is ambiguous.  A cutoff
  (retrieve_clusters keeps a node when dist <= cutoff,
  hierarchical.rs:136-169) is ambiguous for a run when some merge distance
  lies within the largest working-matrix difference (delta) of it.
* OPTICS (optics.rs:51-148): an instance is ambiguous when some pair's oracle
  distance lies within that pair's engine error of eps (the neighbour test
  d <= eps, points_set.rs:150-169, could go the other way).

Every non-ambiguous instance must give the same partition.  The ambiguous
ones are excluded, printed and counted, and must stay a minority.  The
engine's own clustering of its matrix (host and GPU) must also take exactly
the oracle restatement's merges for that matrix.
"""
import numpy as np
import pytest

from bioshell_gb300 import clustering as K
from bioshell_gb300 import synth
from bioshell_gb300.crmsd import CrmsdMatrix
from oracle import clustering as C

pytestmark = pytest.mark.gpu

RULES = ["single", "complete", "average", "median", "centroid", "ward"]
CUT_QUANTILES = (0.5, 0.9, 0.98)  # cutoffs placed between consecutive merge distances
TOL = 1e-4


def _square(tri, n):
    sq = np.zeros((n, n))
    iu = np.triu_indices(n, 1)
    sq[iu] = tri
    return sq + sq.T


def _canonical(labels):
    """Partition labels renumbered by first appearance."""
    seen = {}
    return np.array([seen.setdefault(int(v), len(seen)) for v in labels], dtype=np.int64)


@pytest.fixture(scope="module")
def matrices(engine, oracle_mod):
    x = synth.PLAIN_CPU.generate()
    n = x.shape[0]
    ref = oracle_mod.crmsd_all_vs_all(x)
    got = engine.all_vs_all(x).values.copy()
    err = float(np.abs(got - ref).max())
    assert err <= TOL
    return n, got, ref, err


def test_hierarchical_labels_all_rules(engine, matrices):
    n, got, ref, err = matrices
    sq_eng = _square(got, n).astype(np.float32)
    sq_ref = _square(ref, n).astype(np.float32)
    tri32 = CrmsdMatrix(n, got.astype(np.float32), "triangle")
    total = flagged = 0
    for rule in RULES:
        (ma, da), (mb, db), split, delta, slack = C.lockstep(sq_eng, sq_ref, rule)
        # the engine clusters its own matrix exactly as the restatement does
        host = K.hierarchical_clustering(tri32, rule)
        dev = K.hierarchical_clustering(tri32, rule, engine=engine)
        for t in (host, dev):
            np.testing.assert_array_equal(t.merges, ma)
            np.testing.assert_array_equal(t.dist, da)
        near = slack <= 0.0
        if split is not None:
            assert near[split], f"{rule}: runs part at merge {split} with slack {slack[split]} > 0"
        run_amb = bool(np.any(near))
        dmax = float(delta.max()) if delta.size else 0.0
        srt = np.sort(db.astype(np.float64))
        for q in CUT_QUANTILES:
            k = int(q * (n - 1))
            cut = float(np.float32(0.5 * (srt[k - 1] + srt[k])))
            cut_amb = bool(np.any(np.abs(db.astype(np.float64) - cut) <= dmax)) or \
                bool(np.any(np.abs(da.astype(np.float64) - cut) <= dmax))
            la = _canonical(K.cut_tree(host, cut))
            lb = _canonical(C.cut_labels(n, mb, db, cut))
            same = bool(np.array_equal(la, lb))
            total += 1
            amb = run_amb or cut_amb
            print(f"{rule:9s} cut {cut:8.4f}: clusters {la.max() + 1:4d}  same {same}  "
                  f"ambiguous {amb} (merge margin {run_amb}, cutoff {cut_amb}); "
                  f"least slack {slack.min():.2e}, max delta {dmax:.2e}")
            if amb:
                flagged += 1
            else:
                assert same, f"{rule} at cutoff {cut}: labels differ with no decision within tolerance"
    print(f"hierarchical: {total - flagged} of {total} instances compared, {flagged} excluded as ambiguous "
          f"(engine vs FP64 oracle max |dRMSD| {err:.2e} A)")
    assert flagged <= total // 3


@pytest.mark.parametrize("eps,min_points", [(2.0, 5), (3.0, 10), (4.0, 20)])
def test_optics_labels(matrices, eps, min_points):
    n, got, ref, err = matrices
    sq_ref = _square(ref, n)
    order, reach, cl = K.optics(CrmsdMatrix(n, got, "triangle"), eps, min_points)
    o2, r2, c2 = C.optics(n, lambda i, j: sq_ref[i, j], eps, min_points)
    want = np.zeros(n, dtype=np.int64)
    for k, c in enumerate(c2):
        want[c] = k
    amb = bool(np.any(np.abs(ref - eps) <= np.abs(got - ref)))
    same = bool(np.array_equal(_canonical(cl), _canonical(want)))
    print(f"OPTICS eps {eps} min_points {min_points}: clusters {len(c2)}  same {same}  ambiguous {amb}  "
          f"same order {list(order) == o2}")
    if not amb:
        assert same
        # reachabilities of the same visit order agree within the distance error
        if list(order) == o2:
            r2o = np.array([r2[k] for k in o2])
            assert np.abs(reach - r2o).max() <= TOL
