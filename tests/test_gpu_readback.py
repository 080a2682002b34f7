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
