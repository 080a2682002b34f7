"""TSV export straight from a device-resident crmsd triangle: the streamed
(device -> pinned host, formatted on all host threads) file equals the one
written from the same values in host memory."""
import numpy as np
import pytest

from bioshell_gb300 import formats as F
from bioshell_gb300 import synth

pytestmark = pytest.mark.gpu


def test_tsv_from_device_equals_host(engine, tmp_path):
    import torch
    rng = np.random.default_rng(11)
    x = synth.decoys(synth.base_chain(60, rng), 1500, rng)
    n = x.shape[0]
    dev = torch.empty(n * (n - 1) // 2, dtype=torch.float64, device="cuda")
    engine.all_vs_all(torch.from_numpy(x).cuda(), out=dev)
    host = dev.cpu().numpy()
    labels = [f"model_{i}" for i in range(n)]
    pd, ph = str(tmp_path / "d.tsv"), str(tmp_path / "h.tsv")
    F.write_tsv(pd, dev, labels, n=n)
    F.write_tsv(ph, host, labels, n=n)
    assert open(pd, "rb").read() == open(ph, "rb").read()
    labs, m = F.read_tsv(pd)
    assert labs == labels
    # 6 decimals, then f32: within half a unit of the 6th decimal plus an f32 rounding
    np.testing.assert_allclose(m.values, host, rtol=1.2e-7, atol=5.0001e-7)
