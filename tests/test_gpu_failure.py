"""Failure detection on the GPU without faulting it: each failure is made on
the host or through a kernel argument, and each test checks the status that
comes back and that the context (or server) computes correctly afterwards.

* A device-side wait that runs out: the grid barriers of the GPU
  hierarchical clustering get a 1 ns bound (bs_debug_set_wait_limit, a
  kernel argument); the first barrier wait that outlasts it makes every
  block return, the call returns BS_ERR_TIMEOUT, and with the default bound
  restored the same context clusters correctly.  The same bound on the
  mbarrier waits of the all-vs-all tensor-core kernel's copy and MMA
  threads: the first such wait that is not already complete runs out, every
  role of every block
  stops (copies and MMAs in flight are let complete, tensor memory is
  freed), the call returns BS_ERR_TIMEOUT, and the next call of the same
  context, default bound restored, gives the same matrix bit for bit.
* A failed device allocation: bs_debug_fail_alloc makes a chosen workspace
  allocation of a fresh context fail as out of memory (BS_ERR_OOM); the next
  call, hook disarmed, completes.
* A cancelled request: a query queued behind a clustering job on a
  one-slot server is cancelled; its wait returns BS_ERR_CANCELLED and the
  other requests complete with the results they get alone.
"""
import ctypes

import numpy as np
import pytest

from bioshell_gb300 import CrmsdServer, synth
from bioshell_gb300 import clustering as K
from bioshell_gb300.crmsd import CrmsdMatrix, Engine
from bioshell_gb300.lib import CrmsdError

pytestmark = pytest.mark.gpu

BS_ERR_OOM, BS_ERR_TIMEOUT, BS_ERR_CANCELLED = 3, 4, 10


def _points_matrix(n, seed):
    rng = np.random.default_rng(seed)
    pts = rng.normal(size=(n, 3)) * 4.0
    sq = np.linalg.norm(pts[:, None] - pts[None], axis=2)
    return CrmsdMatrix(n, np.ascontiguousarray(sq[np.triu_indices(n, 1)], dtype=np.float32), "triangle")


def test_barrier_wait_runs_out_and_context_recovers(engine, enginelib):
    m = _points_matrix(600, 3)
    assert enginelib.bs_debug_set_wait_limit(engine._h, 1) == 0
    try:
        with pytest.raises(CrmsdError) as ei:
            K.hierarchical_clustering(m, "average", engine=engine)
        assert ei.value.status == BS_ERR_TIMEOUT
        assert "timed out" in str(ei.value)
    finally:
        assert enginelib.bs_debug_set_wait_limit(engine._h, 0) == 0
    dev = K.hierarchical_clustering(m, "average", engine=engine)
    host = K.hierarchical_clustering(m, "average")
    np.testing.assert_array_equal(dev.merges, host.merges)
    np.testing.assert_array_equal(dev.dist, host.dist)


def test_pipeline_wait_runs_out_and_context_recovers(engine, enginelib, oracle_mod):
    rng = np.random.default_rng(13)
    x = synth.decoys(synth.base_chain(64, rng), 1500, rng, near_dup_frac=0.05)
    before = engine.all_vs_all(x).values.copy()  # a graph captured with the default bound
    assert enginelib.bs_debug_set_wait_limit(engine._h, 1) == 0
    try:
        for _ in range(2):  # graph captured with the 1 ns bound, then replayed
            with pytest.raises(CrmsdError) as ei:
                engine.all_vs_all(x)
            assert ei.value.status == BS_ERR_TIMEOUT
            assert "timed out" in str(ei.value)
    finally:
        assert enginelib.bs_debug_set_wait_limit(engine._h, 0) == 0
    after = engine.all_vs_all(x).values
    np.testing.assert_array_equal(after, before)
    assert engine.metrics()["graph"] == 2  # the default-bound graph, replayed
    assert np.abs(after - oracle_mod.crmsd_all_vs_all(x)).max() <= 1e-4


def test_injected_allocation_failure(enginelib, oracle_mod):
    rng = np.random.default_rng(9)
    x = synth.decoys(synth.base_chain(70, rng), 120, rng)
    ref = oracle_mod.crmsd_all_vs_all(x)
    for after in (0, 2):
        eng = Engine(0)  # fresh: every workspace still has to be allocated
        assert enginelib.bs_debug_fail_alloc(eng._h, after) == 0
        with pytest.raises(CrmsdError) as ei:
            eng.all_vs_all(x)
        assert ei.value.status == BS_ERR_OOM
        assert "bs_debug_fail_alloc" in str(ei.value)
        assert enginelib.bs_debug_fail_alloc(eng._h, -1) == 0
        assert np.abs(eng.all_vs_all(x).values - ref).max() <= 1e-4
        eng.close()
    assert enginelib.bs_debug_fail_alloc(None, 0) == 1
    assert enginelib.bs_debug_set_wait_limit(None, 5) == 1


def test_cancel_queued_request():
    rng = np.random.default_rng(21)
    lib = {64: synth.decoys(synth.base_chain(64, rng), 3000, rng, sigma=(0.3, 3.0))}
    q = synth.decoys(synth.base_chain(64, rng), 24, rng, sigma=(0.3, 3.0))
    job = synth.decoys(synth.base_chain(64, rng), 3000, rng, sigma=(0.3, 3.0))
    srv = CrmsdServer(lib, top_k=10, max_inflight=1)
    try:
        alone = [srv.wait(srv.submit(q[k:k + 8])) for k in (0, 8, 16)]
        tc = srv.submit_cluster(job, 3.0, 5)  # occupies the only slot for a while
        t = [srv.submit(q[k:k + 8]) for k in (0, 8, 16)]
        assert srv.cancel(t[1]) is True
        with pytest.raises(CrmsdError) as ei:
            srv.wait(t[1])
        assert ei.value.status == BS_ERR_CANCELLED
        for k in (0, 2):
            idx, val = srv.wait(t[k])
            np.testing.assert_array_equal(idx, alone[k][0])
            np.testing.assert_array_equal(val, alone[k][1])
        assert srv.wait_cluster(tc).shape == (3000,)
        # a finished request is not cancelled and keeps its result; a ticket
        # already collected, or unknown, is an error
        done = srv.submit(q[:8])
        while not srv.poll(done):
            pass
        assert srv.cancel(done) is False
        idx, val = srv.wait(done)
        np.testing.assert_array_equal(idx, alone[0][0])
        with pytest.raises(CrmsdError):
            srv.cancel(done)
        c = ctypes.c_int32(7)
        assert srv._lib.bs_server_cancel(srv._h, 10 ** 9, ctypes.byref(c)) == 1
    finally:
        srv.close()
