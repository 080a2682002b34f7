"""GPU parity of the crmsd engine against the FP64 oracle, through the C ABI.

Tolerances (Angstrom, |RMSD_gpu - RMSD_oracle|):
  * plain FP64 path: 1e-9 (same method, FP64 throughout);
  * mixed path: 1e-4, the project's accuracy bar.  By default the engine
    certifies 1e-4 per pair: grid quantisation (sqrt(3) 2^e) plus the
    fast path's arithmetic bound, with exact recomputation of any pair whose
    bound does not fit.
Tensor-core exactness is checked bit for bit: the raw TMEM level sums of a
tile must equal the CUDA-core integer sums.
"""
import numpy as np
import pytest

from bioshell_gb300 import synth
from bioshell_gb300.crmsd import CrmsdOptions

pytestmark = pytest.mark.gpu

TOL_MIXED = 1e-4
TOL_PLAIN = 1e-9
# FP64 cancellation floor of G_a + G_b - 2 lambda for (near-)identical pairs:
# ~sqrt(eps (G_a + G_b) / L), about 1e-6 A; the CPU oracle has the same floor
PLAIN_FLOOR = 2e-6


def plain_close(got, ref):
    d = np.abs(np.asarray(got) - ref)
    return bool(np.all(np.where(ref > 1e-3, d <= TOL_PLAIN, d <= PLAIN_FLOOR)))


def _tri_pairs(n, t):
    t = np.asarray(t, dtype=np.int64)
    i = np.floor((2 * n - 1 - np.sqrt((2 * n - 1) ** 2 - 8 * t.astype(np.float64))) / 2).astype(np.int64)
    i = np.where(i * n - i * (i + 1) // 2 > t, i - 1, i)
    i = np.where((i + 1) * n - (i + 1) * (i + 2) // 2 <= t, i + 1, i)
    j = t - (i * n - i * (i + 1) // 2) + i + 1
    return i, j


def test_tensor_core_level_sums_are_exact(engine):
    rng = np.random.default_rng(11)
    x = synth.decoys(synth.base_chain(77, rng), 40, rng, near_dup_frac=0.1)
    tl = engine.debug_tile_levels(x)  # tiles (rows 0..39) x (columns 0..19, 20..39)
    ia, ja = np.meshgrid(np.arange(40), np.arange(40), indexing="ij")
    ia, ja = ia.ravel(), ja.ravel()
    pl, _ = engine.debug_pair_levels(x, ia, ja)

    def row(s, c):  # structures 0-4 of a 32-row group at rows 0-14, 5-9 at rows 16-30
        return 32 * (s // 10) + 3 * (s % 10) + (1 if s % 10 >= 5 else 0) + c

    rows = np.array([[row(s, c) for c in range(3)] for s in range(40)])
    for t in range(len(ia)):
        i, j = ia[t], ja[t]
        if i == j:
            continue
        blk = tl[:, rows[i]][:, :, rows[j]].reshape(4, 9)
        np.testing.assert_array_equal(blk, pl[t])
    assert np.abs(tl).max() < 2 ** 24


def test_config_500x64_all_pairs(engine, oracle_mod):
    x = synth.PLAIN_CPU.generate()
    ref = oracle_mod.crmsd_all_vs_all(x)
    mixed = engine.all_vs_all(x).values
    d = np.abs(mixed - ref)
    print(f"mixed 500x64: max {d.max():.3e} p99 {np.percentile(d, 99):.3e}")
    assert d.max() <= TOL_MIXED
    m = engine.metrics()
    assert 0.0 < m["quant_bound"] < TOL_MIXED
    plain = engine.all_vs_all(x, CrmsdOptions(precision="plain64")).values
    assert plain_close(plain, ref)


def test_golden_fixtures(engine, golden_small, golden_2jqb):
    for x, ref in ((golden_small["xyz"], golden_small["rmsd"]),
                   (golden_2jqb["all_atoms"], golden_2jqb["rmsd_all"]),
                   (golden_2jqb["ca"], golden_2jqb["rmsd_ca"])):
        assert np.abs(engine.all_vs_all(x).values - ref).max() <= TOL_MIXED
        assert plain_close(engine.all_vs_all(x, CrmsdOptions(precision="plain64")).values, ref)


@pytest.mark.parametrize("n,L", [(2, 3), (3, 4), (39, 5), (40, 17), (41, 64), (81, 129), (123, 255), (47, 301)])
def test_ragged_shapes(engine, oracle_mod, n, L):
    rng = np.random.default_rng(n * 1000 + L)
    x = synth.decoys(synth.base_chain(L, rng), n, rng, near_dup_frac=0.1)
    ref = oracle_mod.crmsd_all_vs_all(x)
    assert np.abs(engine.all_vs_all(x).values - ref).max() <= TOL_MIXED
    assert plain_close(engine.all_vs_all(x, CrmsdOptions(precision="plain64")).values, ref)


@pytest.mark.parametrize("L", [420, 560, 700, 900, 1200])
def test_mid_length_chains(engine, oracle_mod, L):
    """Chains where the whole chain's level sums no longer fit the exact
    range: the half layout (every level accumulated per half of the chain,
    both TMEM buffers, one MMA for several levels) and, beyond its reach, the
    long layout.  Near-duplicates included; every pair within the tolerance
    of the oracle and the same matrix from the batched call.  Up to 900 atoms
    few pairs are recomputed exactly; at 1,200 atoms level 1 no longer fits
    in halves of the chain, the coarser relaxed grid is chosen, and its
    quantisation leaves the pairs to the exact recomputation."""
    rng = np.random.default_rng(L + 7)
    x = synth.decoys(synth.base_chain(L, rng), 81, rng, near_dup_frac=0.1)
    got = engine.all_vs_all(x).values.copy()
    assert engine.metrics()["pairs_plain"] == 0
    if L <= 900:
        assert engine.metrics()["pairs_refined"] <= 0.05 * got.size
    assert np.abs(got - oracle_mod.crmsd_all_vs_all(x)).max() <= TOL_MIXED
    np.testing.assert_array_equal(engine.batched([x])[0].values, got)


@pytest.mark.parametrize("L", [1500, 4096, 16384])
def test_very_long_chains(engine, oracle_mod, L):
    """Chains up to the limit of 16,384 atoms (the preparation's 32-bit
    digit-norm sums cannot overflow below it).  At 1,500 atoms the mixed path
    still runs (on a grid coarse enough for its exact levels, with exact
    recomputation where the certified bound does not fit).  Beyond
    ~3,000 atoms the digit-1 products exceed the exact range even in quarters
    of the chain, no coordinate grid fits, and the set is computed on the
    plain FP64 GPU path instead (metrics: pairs_plain).  A row-ranged call of
    such a set reports BS_ERR_UNSUPPORTED (the plain path writes every row);
    one atom beyond the limit is rejected before any GPU work."""
    from bioshell_gb300.lib import CrmsdError
    rng = np.random.default_rng(L)
    x = synth.decoys(synth.base_chain(L, rng), 41, rng, near_dup_frac=0.1)
    got = engine.all_vs_all(x).values
    ref = oracle_mod.crmsd_all_vs_all(x)
    plain = engine.metrics()["pairs_plain"]
    if L == 1500:
        assert plain == 0
        assert np.abs(got - ref).max() <= TOL_MIXED
    else:
        assert plain == 41 * 40 // 2
        # FP64 against FP64: the cancellation floor of G_a + G_b - 2 lambda
        # grows with the chain's extent (coordinates up to ~1,200 A here)
        assert np.abs(got - ref).max() <= 1e-6
        with pytest.raises(CrmsdError) as ei:
            engine.all_vs_all(x, CrmsdOptions(rows=(0, 40)))
        assert ei.value.status == 5
    if L == 16384:
        with pytest.raises(CrmsdError) as ei:
            engine.all_vs_all(np.zeros((2, L + 1, 3)))
        assert ei.value.status == 5


def test_far_and_lopsided_coordinates(engine, oracle_mod):
    """Structures up to 30,000 A from the origin (inside the fixed-point range
    of 2^15 A), of different sizes in one set, and lopsided ones whose
    centroid lies far from the middle of their extent (one atom 200 A out):
    the centring, the grid choice and the digits must stay within tolerance
    of the FP64 oracle on every pair."""
    rng = np.random.default_rng(29)
    x = synth.decoys(synth.base_chain(270, rng), 48, rng, near_dup_frac=0.1)
    x += rng.uniform(-30000.0, 30000.0, size=(48, 1, 3))
    x[3:9, 17] += np.array([200.0, -150.0, 90.0])  # one atom far out in six structures
    c = x[20:24].mean(axis=1, keepdims=True)
    x[20:24] = c + 1.5 * (x[20:24] - c)  # larger structures in the same set
    ref = oracle_mod.crmsd_all_vs_all(x)
    assert np.abs(engine.all_vs_all(x).values - ref).max() <= TOL_MIXED
    assert plain_close(engine.all_vs_all(x, CrmsdOptions(precision="plain64")).values, ref)


def test_duplicates_and_rigid_copies(engine, oracle_mod):
    rng = np.random.default_rng(5)
    x = synth.decoys(synth.base_chain(300, rng), 60, rng, sigma=(0.2, 2.0))
    rot = synth.random_rotations(10, rng)
    extra = [x[k] @ rot[k].T + rng.uniform(-40, 40, 3) for k in range(10)] + [x[k].copy() for k in range(10)]
    x = np.concatenate([x, np.stack(extra)])
    ref = oracle_mod.crmsd_all_vs_all(x)
    got = engine.all_vs_all(x).values
    assert np.abs(got - ref).max() <= TOL_MIXED
    assert engine.metrics()["pairs_refined"] >= 20


def test_layouts_and_types(engine, oracle_mod, golden_small):
    x = golden_small["xyz"]
    n = x.shape[0]
    ref = golden_small["rmsd"]
    sq = engine.all_vs_all(x, CrmsdOptions(layout="square")).to_square()
    iu = np.triu_indices(n, 1)
    assert np.all(np.diag(sq) == 0.0)
    np.testing.assert_array_equal(sq, sq.T)
    assert np.abs(sq[iu] - ref).max() <= TOL_MIXED
    f32 = engine.all_vs_all(x, CrmsdOptions(out_type="f32"))
    assert f32.values.dtype == np.float32
    assert np.abs(f32.values - ref).max() <= TOL_MIXED + 1e-5
    sqp = engine.all_vs_all(x, CrmsdOptions(layout="square", precision="plain64", out_type="f32")).to_square()
    assert np.abs(sqp[iu] - ref).max() <= 1e-5


def test_pairs_api_and_single_pair(engine, oracle_mod):
    x = synth.Workload("p", n=900, L=150, seed=21, near_dup_frac=0.05).generate()
    rng = np.random.default_rng(2)
    ii = rng.integers(0, 900, 20000)
    jj = rng.integers(0, 900, 20000)
    ref = oracle_mod.crmsd_pairs(x, ii, jj)
    got = engine.pairs(x, ii, jj, CrmsdOptions(precision="mixed"))
    assert np.abs(got - ref).max() <= TOL_MIXED
    assert plain_close(engine.pairs(x, ii, jj, CrmsdOptions(precision="plain64")), ref)
    assert abs(engine.crmsd(x[0], x[1]) - oracle_mod.crmsd(x[0], x[1])) <= TOL_MIXED
    assert engine.crmsd(x[3], x[3]) <= TOL_MIXED


def test_subsample_20000x150(engine, oracle_mod):
    """20,000 x 150 decoys: every pair on the GPU, 1e6 seeded pairs checked."""
    w = synth.PLAIN_FP64_GPU
    x = w.generate()
    n = w.n
    sel = np.random.default_rng(123).choice(n * (n - 1) // 2, 1000000, replace=False)
    i, j = _tri_pairs(n, sel)
    ref = oracle_mod.crmsd_pairs(x, i, j)
    mixed = engine.all_vs_all(x).values
    assert np.abs(mixed[sel] - ref).max() <= TOL_MIXED
    plain = engine.all_vs_all(x, CrmsdOptions(precision="plain64")).values
    assert plain_close(plain[sel], ref)
    # size-independent properties of the full matrix
    assert np.all(np.isfinite(mixed)) and mixed.min() >= 0.0
    assert np.abs(mixed - plain).max() <= TOL_MIXED


def test_deterministic(engine, golden_2jqb):
    x = golden_2jqb["all_atoms"]
    a = engine.all_vs_all(x).values.copy()
    b = engine.all_vs_all(x).values
    np.testing.assert_array_equal(a, b)


def test_device_pointers(engine, golden_small):
    torch = pytest.importorskip("torch")
    x = torch.from_numpy(golden_small["xyz"]).cuda()
    n = x.shape[0]
    out = torch.empty(n * (n - 1) // 2, dtype=torch.float64, device="cuda")
    engine.all_vs_all(x, out=out)
    torch.cuda.synchronize()
    assert np.abs(out.cpu().numpy() - golden_small["rmsd"]).max() <= TOL_MIXED


def test_row_ranges_partition_the_matrix(engine, oracle_mod):
    """Row ranges (bs_opts.row_begin/row_end): three ranges from
    bs_partition_rows, written into one host buffer, give the full call's
    result bit for bit; a single range leaves every element outside it as it
    was; bad ranges are rejected.  One range per GPU partitions an
    all-vs-all with no exchange between them."""
    from bioshell_gb300.crmsd import partition_rows
    from bioshell_gb300.lib import CrmsdError
    rng = np.random.default_rng(55)
    x = synth.decoys(synth.base_chain(90, rng), 1000, rng, near_dup_frac=0.1)
    n = x.shape[0]
    full = engine.all_vs_all(x).values.copy()
    b = partition_rows(n, 3)
    out = np.full(n * (n - 1) // 2, -7.0)
    for p in range(3):
        engine.all_vs_all(x, CrmsdOptions(rows=(int(b[p]), int(b[p + 1]))), out=out)
    np.testing.assert_array_equal(out, full)
    # one range alone: the rest untouched, pinned and device outputs too
    lo, hi = int(b[1]), int(b[2])
    e0, e1 = lo * n - lo * (lo + 1) // 2, hi * n - hi * (hi + 1) // 2
    oh = engine.host_empty((n * (n - 1) // 2,), np.float64)
    oh[...] = -7.0
    engine.all_vs_all(x, CrmsdOptions(rows=(lo, hi)), out=oh)
    assert engine.metrics()["pairs"] == e1 - e0
    np.testing.assert_array_equal(oh[e0:e1], full[e0:e1])
    assert np.all(oh[:e0] == -7.0) and np.all(oh[e1:] == -7.0)
    assert np.abs(full[e0:e1] - oracle_mod.crmsd_all_vs_all(x)[e0:e1]).max() <= TOL_MIXED
    for bad in ((1, 80), (40, 81), (80, 40), (0, n + 40)):
        with pytest.raises(CrmsdError) as ei:
            engine.all_vs_all(x, CrmsdOptions(rows=bad))
        assert ei.value.status == 1
    with pytest.raises(CrmsdError) as ei:
        engine.all_vs_all(x, CrmsdOptions(rows=(0, 80), precision="plain64"))
    assert ei.value.status == 5
