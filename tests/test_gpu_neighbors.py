"""eps-neighbour lists on the GPU (bs_neighbors): the sparse form of the
all-vs-all that OPTICS consumes (NeighborsOf, points_set.rs:29-39).

* Against the FP64 oracle: row i holds every j != i whose oracle distance
  (rounded to f32, as the reference stores it) is <= eps -- the rule of
  CartesianPoints::neighbors_of (points_set.rs:150-169) without the point
  itself -- with distances within the 1e-4 A tolerance, ordered by (d, j).
  Rows where some distance lies within the tolerance of eps are skipped and
  counted.
* The lists equal those read off the dense f32 matrix of the same call path:
  the same (j, d) entries per row, ordered by (d, j), bit for bit.
* OPTICS over the lists gives the dense matrix's order, reachability and
  labels.
* Rows longer than the shared-memory sort (4096 entries) take the merge path.
"""
import numpy as np
import pytest

from bioshell_gb300 import clustering as K
from bioshell_gb300 import synth
from bioshell_gb300.crmsd import CrmsdOptions
from bioshell_gb300.lib import CrmsdError

pytestmark = pytest.mark.gpu


def _dense_f32(engine, x):
    m = engine.all_vs_all(x, CrmsdOptions(out_type="f32", layout="square"))
    return np.asarray(m.values, dtype=np.float32).reshape(x.shape[0], x.shape[0])


def _check_equal(engine, x, eps):
    rp, col, dist = engine.neighbors(x, eps)
    sq = _dense_f32(engine, x)
    rp2, col2, dist2 = K.neighbors_from_dense(sq, eps)
    np.testing.assert_array_equal(rp, rp2)
    np.testing.assert_array_equal(col, col2)
    np.testing.assert_array_equal(dist, dist2)
    return rp, col, dist, sq


TOL = 1e-4


@pytest.mark.parametrize("eps", [0.8, 2.5, 6.0])
def test_lists_match_the_oracle(engine, oracle_mod, eps):
    rng = np.random.default_rng(15)
    x = synth.decoys(synth.base_chain(120, rng), 700, rng, sigma=(0.2, 4.0), near_dup_frac=0.05)
    x[10] = x[11]  # identical structures: distance 0
    n = x.shape[0]
    ref = np.zeros((n, n))
    ref[np.triu_indices(n, 1)] = oracle_mod.crmsd_all_vs_all(x)
    ref = ref + ref.T
    ref32 = ref.astype(np.float32)
    rp, col, dist = engine.neighbors(x, eps)
    skipped = 0
    for i in range(n):
        others = np.arange(n) != i
        if np.any(np.abs(ref[i, others] - eps) <= TOL):
            skipped += 1  # a neighbour decision within tolerance of eps
            continue
        want = np.flatnonzero((ref32[i] <= eps) & others)
        c, d = col[rp[i]:rp[i + 1]], dist[rp[i]:rp[i + 1]]
        np.testing.assert_array_equal(np.sort(c), want)
        assert np.all(np.abs(d.astype(np.float64) - ref[i, c]) <= TOL)
        # ordered by (d, j) on the engine's values
        o = np.lexsort((c, d))
        np.testing.assert_array_equal(o, np.arange(c.size))
    print(f"eps {eps}: {n - skipped} rows compared, {skipped} skipped (a distance within {TOL} A of eps), "
          f"{rp[-1]} entries")
    assert skipped <= n // 10


@pytest.mark.parametrize("eps", [0.8, 2.5, 6.0])
def test_lists_equal_dense_rows(engine, eps):
    rng = np.random.default_rng(5)
    base = synth.base_chain(120, rng)
    x = synth.decoys(base, 700, rng, sigma=(0.2, 4.0), near_dup_frac=0.05)
    x[10] = x[11]  # identical structures: distance 0 ties
    _check_equal(engine, x, eps)


def test_optics_from_lists_equals_dense(engine):
    rng = np.random.default_rng(6)
    parts = [synth.decoys(synth.base_chain(90, rng), 150, rng, sigma=(0.3, 2.5)) for _ in range(3)]
    x = np.concatenate(parts)
    eps, mp = 3.0, 5
    rp, col, dist, sq = _check_equal(engine, x, eps)
    n = x.shape[0]
    iu = np.triu_indices(n, 1)
    from bioshell_gb300.crmsd import CrmsdMatrix
    m = CrmsdMatrix(n, np.ascontiguousarray(sq[iu]), "triangle")
    o1, r1, c1 = K.optics(m, eps, mp)
    o2, r2, c2 = K.optics_neighbors(rp, col, dist, eps, mp)
    np.testing.assert_array_equal(o1, o2)
    np.testing.assert_array_equal(r1, r2)
    np.testing.assert_array_equal(c1, c2)


def test_long_rows_take_the_merge_path(engine):
    rng = np.random.default_rng(7)
    x = synth.decoys(synth.base_chain(48, rng), 4700, rng, sigma=(0.5, 2.0))
    rp, col, dist = engine.neighbors(x, 1e6)  # every pair: rows of 4699 entries
    n = x.shape[0]
    assert rp[-1] == n * (n - 1)
    sq = _dense_f32(engine, x)
    for i in (0, 1, 2345, n - 1):
        j = np.flatnonzero(np.arange(n) != i)
        o = np.lexsort((j, sq[i, j]))
        np.testing.assert_array_equal(col[rp[i]:rp[i + 1]], j[o])
        np.testing.assert_array_equal(dist[rp[i]:rp[i + 1]], sq[i, j[o]])


def test_small_and_degenerate(engine):
    rng = np.random.default_rng(8)
    for n in (0, 1):
        rp, col, dist = engine.neighbors(np.zeros((n, 10, 3)) if n == 0 else rng.normal(size=(n, 10, 3)), 1.0)
        assert rp.tolist() == [0] * (n + 1) and col.size == 0
    x = synth.decoys(synth.base_chain(30, rng), 2, rng)
    x[1] = x[0]
    rp, col, dist = engine.neighbors(x, 1e-6)  # identical structures only
    assert rp.tolist() == [0, 1, 2] and col.tolist() == [1, 0] and np.all(dist <= 1e-6)
    with pytest.raises(CrmsdError) as e:
        engine.neighbors(x, 1.0, CrmsdOptions(precision="plain64"))
    assert e.value.status == 5
