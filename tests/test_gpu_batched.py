"""Batched all-vs-all (bs_batched) on the GPU: many decoy sets of uneven size
and chain length in one persistent tensor-core launch, replayed as a CUDA
graph for repeated shapes.

Each set gets its own grid and error budget, so a set's result is the same
bit for bit whether it runs alone (bs_all_vs_all) or inside a batch, and
whether the call sequence is captured in a graph or launched directly.
Against the FP64 oracle every value is within the mixed-path tolerance
(1e-4 A).  Per-set OPTICS partitions are compared with the plain FP64
path's: they can only differ through a distance within the |mixed - FP64|
gap of eps, or a border point whose two candidate clusters reach it at
distances within that gap (processing order), both rare at gaps ~1e-5 A.
"""
import numpy as np
import pytest

from bioshell_gb300 import clustering as K
from bioshell_gb300 import synth
from bioshell_gb300.crmsd import CrmsdOptions

pytestmark = pytest.mark.gpu

TOL_MIXED = 1e-4


def _sets(seed, shapes, sigma_range=(0.2, 6.0)):
    rng = np.random.default_rng(seed)
    out = []
    for n, L in shapes:
        base = synth.base_chain(L, rng)
        out.append(synth.decoys(base, n, rng, sigma=sigma_range, near_dup_frac=0.05))
    return out


SHAPES = [(45, 40), (2, 64), (1, 30), (130, 150), (61, 800), (97, 257), (0, 12), (300, 64), (21, 401)]


def test_batched_matches_single_set_calls_bit_for_bit(engine):
    sets = _sets(3, SHAPES)
    mats = engine.batched(sets)
    for x, m in zip(sets, mats):
        if x.shape[0] < 2:
            assert m.values.size == 0
            continue
        alone = engine.all_vs_all(x).values
        np.testing.assert_array_equal(m.values, alone)


def test_batched_against_oracle(engine, oracle_mod):
    sets = _sets(4, SHAPES)
    mats = engine.batched(sets)
    worst = 0.0
    for x, m in zip(sets, mats):
        if x.shape[0] < 2:
            continue
        ref = oracle_mod.crmsd_all_vs_all(x)
        worst = max(worst, float(np.abs(m.values - ref).max()))
    print(f"batched max |d| vs oracle {worst:.3e}")
    assert worst <= TOL_MIXED


def test_long_chains_800_atoms(engine, oracle_mod):
    rng = np.random.default_rng(8)
    x = synth.decoys(synth.base_chain(800, rng), 48, rng, near_dup_frac=0.1)
    got = engine.all_vs_all(x).values
    m = engine.metrics()
    ref = oracle_mod.crmsd_all_vs_all(x)
    assert np.abs(got - ref).max() <= TOL_MIXED
    assert m["quant_bound"] < TOL_MIXED
    # levels 1 and 2 are accumulated in parts of the chain, so levels 0-2 stay
    # exact; only level 3's bounded rounding can send a near-duplicate pair
    # to the exact recomputation
    assert m["pairs_refined"] <= 0.02 * len(got)


def test_graph_replay_equals_direct_launches(engine):
    shapes = [(70, 100), (33, 310), (150, 48)]
    a, b = _sets(5, shapes), _sets(6, shapes)
    direct_a = [m.values for m in engine.batched(a, CrmsdOptions(graph=False))]
    assert engine.metrics()["graph"] == 0
    first = [m.values for m in engine.batched(a)]
    assert engine.metrics()["graph"] in (1, 2)
    second = [m.values for m in engine.batched(b)]  # same shapes, new coordinates: replay
    assert engine.metrics()["graph"] == 2
    direct_b = [m.values for m in engine.batched(b, CrmsdOptions(graph=False))]
    for u, v in zip(first, direct_a):
        np.testing.assert_array_equal(u, v)
    for u, v in zip(second, direct_b):
        np.testing.assert_array_equal(u, v)


def test_batched_layouts_and_device_buffers(engine):
    torch = pytest.importorskip("torch")
    sets = _sets(7, [(50, 60), (37, 123)])
    tri = engine.batched(sets)
    sq = engine.batched(sets, CrmsdOptions(layout="square", out_type="f32"))
    for t, s in zip(tri, sq):
        np.testing.assert_allclose(s.values.reshape(t.n, t.n), t.to_square().astype(np.float32), rtol=0, atol=0)
    dev_sets = [torch.from_numpy(sets[0]).cuda(), sets[1]]  # one set on the device, one on the host
    outs = [torch.empty(50 * 49 // 2, dtype=torch.float64, device="cuda"), np.empty(37 * 36 // 2)]
    mats = engine.batched(dev_sets, outs=outs)
    np.testing.assert_array_equal(mats[0].values.cpu().numpy(), tri[0].values)
    np.testing.assert_array_equal(mats[1].values, tri[1].values)


def test_batched_plain64_matches_oracle(engine, oracle_mod):
    sets = _sets(9, [(40, 50), (25, 90)])
    mats = engine.batched(sets, CrmsdOptions(precision="plain64"))
    for x, m in zip(sets, mats):
        ref = oracle_mod.crmsd_all_vs_all(x)
        d = np.abs(m.values - ref)
        assert np.all(np.where(ref > 1e-3, d <= 1e-9, d <= 2e-6))


def _partition(cl):
    groups = {}
    for i, c in enumerate(cl):
        groups.setdefault(int(c), []).append(i)
    return sorted(tuple(g) for g in groups.values())


def test_per_set_optics_against_fp64_path(engine):
    shapes = [(120, 60), (200, 150), (90, 420), (150, 45), (60, 700)]
    sets = _sets(10, shapes, sigma_range=(0.2, 6.0))
    mixed = engine.batched(sets)
    plain = engine.batched(sets, CrmsdOptions(precision="plain64"))
    eps, min_points = 3.0, 5
    agree = 0
    for m, p in zip(mixed, plain):
        gap = float(np.abs(m.values - p.values).max())
        assert gap <= TOL_MIXED
        _, _, cm = K.optics(m, eps, min_points)
        _, _, cp = K.optics(p, eps, min_points)
        agree += _partition(cm) == _partition(cp)
    assert agree >= len(shapes) - 1


def test_batched_rejects_bad_sets(engine, oracle_mod):
    from bioshell_gb300.lib import CrmsdError
    x = np.zeros((3, 4, 3))
    x[1, 0, 0] = np.nan
    with pytest.raises(CrmsdError) as e:
        engine.batched([np.ones((5, 6, 3)) * np.arange(6)[None, :, None], x])
    assert e.value.status == 6  # BS_ERR_NONFINITE
    # a set beyond the fixed-point range (|x| >= 32768 A) runs on the plain
    # FP64 path; the other sets of the call stay on the mixed path
    rng = np.random.default_rng(21)
    far = synth.decoys(synth.base_chain(12, rng), 5, rng)
    far[0] += 40000.0
    near = _sets(11, [(30, 20)])[0]
    res = engine.batched([near, far])
    assert engine.metrics()["pairs_plain"] == 10
    assert np.abs(res[1].values - oracle_mod.crmsd_all_vs_all(far)).max() <= 1e-6
    alone = engine.batched([near])[0].values
    np.testing.assert_array_equal(res[0].values, alone)
    # the context stays usable
    ok = engine.batched(_sets(11, [(10, 20)]))
    assert np.all(ok[0].values >= 0)


def test_narrow_tiles_match_wide_bit_for_bit(engine):
    # the same exact integer level sums on 40 x 10 tiles (MMA N = 32)
    sets = _sets(12, [(57, 70), (130, 200), (23, 500), (3, 40)])
    wide = [m.values for m in engine.batched(sets, CrmsdOptions(graph=False))]
    for x in sets:
        engine.set_tile_shape(x.shape[1], x.shape[0], "narrow")
    narrow = engine.batched(sets, CrmsdOptions(graph=False, autotune=True))
    assert engine.metrics()["narrow_jobs"] == len(sets)
    for u, v in zip(wide, narrow):
        np.testing.assert_array_equal(u, v.values)


def test_autotuner_times_each_class_once(engine):
    sets = _sets(13, [(61, 90), (62, 90), (900, 300)])
    engine.batched(sets, CrmsdOptions(autotune=True))
    m = engine.metrics()
    assert 1 <= m["tuned_classes"] <= 2  # the first two sets share a class
    assert engine.tile_shape(90, 61) in ("wide", "narrow")
    again = engine.batched(sets, CrmsdOptions(autotune=True))
    assert engine.metrics()["tuned_classes"] == 0
    for x, mtx in zip(sets, again):
        np.testing.assert_array_equal(mtx.values, engine.all_vs_all(x).values)


def test_tuning_cache_persists_as_json(engine, tmp_path):
    """The autotuner's cache written as JSON (keyed by the SM count) and read
    into a fresh context: the same choices, and no class timed again."""
    from bioshell_gb300.crmsd import Engine
    sets = _sets(17, [(70, 48), (1300, 120)])
    engine.batched(sets, CrmsdOptions(autotune=True))
    path = tmp_path / "tuning.json"
    engine.save_tuning(str(path))
    saved = engine.tuning()
    assert saved["num_sms"] > 0 and len(saved["classes"]) >= 2
    fresh = Engine(0)
    try:
        assert fresh.tuning()["classes"] == []
        assert fresh.load_tuning(str(path))
        assert sorted(map(tuple, fresh.tuning()["classes"])) == sorted(map(tuple, saved["classes"]))
        fresh.batched(sets, CrmsdOptions(autotune=True))
        assert fresh.metrics()["tuned_classes"] == 0
        for x in sets:
            assert fresh.tile_shape(x.shape[1], x.shape[0]) == engine.tile_shape(x.shape[1], x.shape[0])
        # a cache from a GPU of another size is not applied
        import json
        other = json.loads(path.read_text())
        other["num_sms"] += 1
        path.write_text(json.dumps(other))
        assert not Engine(0).load_tuning(str(path))
    finally:
        fresh.close()
