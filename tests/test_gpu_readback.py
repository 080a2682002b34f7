"""Banded read-back: a large triangle written to pinned host memory is copied
band by band while the later bands compute.  The result must equal the
one-shot device result bit for bit, with pairs recomputed exactly inside the
bands, and also when the recomputation queue overflows (the per-band
sentinel scan)."""
import numpy as np
import pytest

from bioshell_gb300 import synth
from bioshell_gb300.crmsd import CrmsdOptions

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def dup_set():
    # 6,000 structures of 24 atoms (17,997,000 pairs, above the banding
    # threshold of 2^24); the last 600 are exact copies of structures spread
    # over the whole set, so flagged pairs fall into many bands
    rng = np.random.default_rng(77)
    base = synth.base_chain(24, rng)
    xs = synth.decoys(base, 5400, rng)
    src = rng.choice(5400, 600, replace=False)
    return np.ascontiguousarray(np.concatenate([xs, xs[src]]))


def _device_result(engine, x, opts):
    import torch

    xd = torch.from_numpy(x).cuda()
    n = x.shape[0]
    out = torch.empty(n * (n - 1) // 2, dtype=torch.float64, device="cuda")
    engine.all_vs_all(xd, opts, out=out)
    torch.cuda.synchronize()
    return out.cpu().numpy(), engine.metrics()


def test_banded_readback_equals_device_result(engine, dup_set):
    x = dup_set
    n = x.shape[0]
    ref, m0 = _device_result(engine, x, CrmsdOptions())
    assert m0["pairs_refined"] >= 600
    assert (ref >= 0).all()
    xh = engine.host_empty(x.shape, np.float64)
    xh[...] = x
    oh = engine.host_empty((n * (n - 1) // 2,), np.float64)
    oh[...] = -7.0
    engine.all_vs_all(xh, CrmsdOptions(), out=oh)
    m1 = engine.metrics()
    assert m1["main_launches"] > 9  # ran in bands
    np.testing.assert_array_equal(oh, ref)
    # pageable host output: one copy at the end, same values
    op = np.full(n * (n - 1) // 2, -7.0)
    engine.all_vs_all(x, CrmsdOptions(), out=op)
    assert engine.metrics()["main_launches"] == 9
    np.testing.assert_array_equal(op, ref)


def test_reused_tile_table_and_bands(engine, dup_set):
    """A context keeps the last call's tile table and read-back bands and
    reuses them for a call of the same shapes.  Calls that alternate shapes,
    row ranges and neighbour lists, and repeat a shape with other
    coordinates, must equal a fresh context's results bit for bit."""
    from bioshell_gb300.crmsd import Engine
    x = dup_set
    n = x.shape[0]
    y = np.ascontiguousarray(x[::-1])  # the same shape, other coordinates in every position
    small = np.ascontiguousarray(x[:777])
    fresh = Engine(0)
    try:
        def ref(z, opts=None):
            return fresh.all_vs_all(z, opts).values.copy()

        ref_x, ref_y, ref_s = ref(x), ref(y), ref(small)
        ref_r = ref(x, CrmsdOptions(rows=(400, 1200)))
        xh = engine.host_empty(x.shape, np.float64)
        oh = engine.host_empty((n * (n - 1) // 2,), np.float64)
        for z, want in ((x, ref_x), (y, ref_y), (small, ref_s), (x, ref_x), (y, ref_y)):
            if z.shape[0] == n:  # pinned in and out: the banded path
                xh[...] = z
                oh[...] = -7.0
                engine.all_vs_all(xh, CrmsdOptions(), out=oh)
                assert engine.metrics()["main_launches"] > 9
                np.testing.assert_array_equal(oh, want)
            else:
                np.testing.assert_array_equal(engine.all_vs_all(z).values, want)
        # a row range of the same n: its own tile table, then the full one again
        e0, e1 = 400 * n - 400 * 401 // 2, 1200 * n - 1200 * 1201 // 2
        xh[...] = x
        oh[...] = -7.0
        engine.all_vs_all(xh, CrmsdOptions(rows=(400, 1200)), out=oh)
        np.testing.assert_array_equal(oh[e0:e1], ref_r[e0:e1])
        engine.all_vs_all(small, CrmsdOptions(rows=(0, 80)))
        engine.neighbors(small, 2.0)
        np.testing.assert_array_equal(engine.all_vs_all(small).values, ref_s)
        xh[...] = y
        engine.all_vs_all(xh, CrmsdOptions(), out=oh)
        np.testing.assert_array_equal(oh, ref_y)
    finally:
        fresh.close()


@pytest.mark.parametrize("pinned", [False, True])
def test_queue_overflow_scan(engine, dup_set, pinned):
    x = dup_set
    n = x.shape[0]
    ref, _ = _device_result(engine, x, CrmsdOptions())
    opts = CrmsdOptions(flag_queue=64)
    if pinned:
        xh = engine.host_empty(x.shape, np.float64)
        xh[...] = x
        out = engine.host_empty((n * (n - 1) // 2,), np.float64)
        out[...] = -7.0
        engine.all_vs_all(xh, opts, out=out)
    else:
        out, m = _device_result(engine, x, opts)
    assert engine.metrics()["pairs_refined"] > 64
    np.testing.assert_array_equal(out, ref)


@pytest.fixture(scope="module")
def many_sets():
    # 12 sets of 1,000-2,400 structures (about 1.9e7 pairs, above the banding
    # threshold) with exact copies inside each set, and chain lengths from 24
    # to 90 atoms so that the tile order (longest chains first) differs from
    # the set order
    rng = np.random.default_rng(78)
    sets = []
    for k in range(12):
        L = int(rng.integers(24, 91))
        n = int(rng.integers(1000, 2401))
        xs = synth.decoys(synth.base_chain(L, rng), n - 40, rng)
        sets.append(np.ascontiguousarray(np.concatenate([xs, xs[rng.choice(n - 40, 40, replace=False)]])))
    return sets


@pytest.mark.parametrize("flag_queue", [0, 64])
def test_batched_banded_readback_equals_device_result(engine, many_sets, flag_queue):
    """Many sets with pinned host outputs: bands end on set boundaries and each
    band's sets are copied while later bands compute (with pinned inputs, each
    band's sets are also uploaded and prepared while earlier bands compute).
    Every set's result
    equals the one-shot result with pageable outputs bit for bit, also when
    the recomputation queue overflows (flag_queue=64: the per-band scan)."""
    opts = CrmsdOptions(flag_queue=flag_queue)
    ref = [m.values.copy() for m in engine.batched(many_sets, opts)]
    assert engine.metrics()["main_launches"] == 9  # pageable outputs: one launch sequence
    hin = []
    for x in many_sets:
        h = engine.host_empty(x.shape, np.float64)
        h[...] = x
        hin.append(h)
    houts = []
    for x in many_sets:
        o = engine.host_empty((x.shape[0] * (x.shape[0] - 1) // 2,), np.float64)
        o[...] = -7.0
        houts.append(o)
    # pinned inputs: each band's sets are uploaded and prepared band by band;
    # pageable inputs: uploaded up front, read back in bands
    for inputs in (hin, many_sets):
        for o in houts:
            o[...] = -7.0
        engine.batched(inputs, opts, outs=houts)
        m = engine.metrics()
        assert m["main_launches"] > 9  # ran in bands
        if flag_queue:
            assert m["pairs_refined"] > flag_queue
        for got, want in zip(houts, ref):
            np.testing.assert_array_equal(got, want)
