"""Serving (bs_server_*) on the GPU: a device-resident library bucketed by
chain length, continuous batching, top-k queries and mixed-in clustering
jobs.

* Top-k: every returned value is within 1e-4 A of the FP64 oracle, and the
  returned indices are the oracle's k nearest except where two library
  structures lie within 2e-4 A of each other at the cut.
* Alone vs mix: a query's result is identical (indices and values, bit for
  bit) when it runs alone and when it is batched with other queries and
  clustering jobs.
* Clustering jobs: OPTICS labels equal those of OPTICS run on the engine's
  own all-vs-all of the same structures.
"""
import threading

import numpy as np
import pytest

from bioshell_gb300 import clustering as K
from bioshell_gb300 import synth
from bioshell_gb300.crmsd import CrmsdOptions
from bioshell_gb300.lib import CrmsdError

pytestmark = pytest.mark.gpu

TOL = 1e-4
TOPK = 20


def _family_library(rng, L, n, families=4):
    parts = []
    for _ in range(families):
        parts.append(synth.decoys(synth.base_chain(L, rng), n // families, rng, sigma=(0.3, 3.0)))
    return np.concatenate(parts), parts


@pytest.fixture(scope="module")
def library():
    rng = np.random.default_rng(77)
    lib64, fam64 = _family_library(rng, 64, 600)
    lib128, fam128 = _family_library(rng, 128, 160)
    return {64: lib64, 128: lib128}, {64: fam64, 128: fam128}, rng


@pytest.fixture(scope="module")
def server(library, enginelib):
    from bioshell_gb300 import CrmsdServer
    lib, _, _ = library
    s = CrmsdServer(lib, top_k=TOPK, max_inflight=3)
    yield s
    s.close()


def _queries(library, L, q, seed):
    _, fams, _ = library
    rng = np.random.default_rng(seed)
    base = fams[L][rng.integers(len(fams[L]))][0]
    return synth.decoys(base - base.mean(axis=0), q, rng, sigma=(0.3, 2.0))


def _check_against_oracle(lib, x, idx, val, oracle_mod):
    n = lib.shape[0]
    for r in range(x.shape[0]):
        pair = np.concatenate([x[r:r + 1], lib])
        ref = oracle_mod.crmsd_pairs(pair, np.zeros(n, dtype=np.int64), np.arange(1, n + 1))
        assert np.all(idx[r] >= 0)
        np.testing.assert_allclose(val[r], ref[idx[r]], rtol=0, atol=TOL)
        order = np.lexsort((np.arange(n), ref))
        kth = ref[order[TOPK - 1]]
        want = set(order[:TOPK][ref[order[:TOPK]] < kth - 2 * TOL].tolist())
        got = set(idx[r].tolist())
        assert want <= got
        assert np.all(np.diff(val[r]) >= 0)


def test_topk_against_oracle(server, library, oracle_mod):
    lib, _, _ = library
    for L, q, seed in ((64, 7, 1), (128, 3, 2), (64, 45, 3)):
        x = _queries(library, L, q, seed)
        idx, val = server.wait(server.submit(x))
        assert idx.shape == (q, TOPK)
        _check_against_oracle(lib[L], x[: min(q, 6)], idx[: min(q, 6)], val[: min(q, 6)], oracle_mod)


def test_same_result_alone_and_in_the_mix(server, library):
    lib, _, rng = library
    probes = [_queries(library, 64, 33, 10), _queries(library, 128, 5, 11), _queries(library, 64, 1, 12)]
    alone = [server.wait(server.submit(x)) for x in probes]
    # now the same queries among concurrent traffic from several threads
    tickets = {}
    others = []

    def noise(seed):
        r = np.random.default_rng(seed)
        for _ in range(6):
            L = 64 if r.random() < 0.7 else 128
            others.append(server.submit(_queries(library, L, int(r.integers(1, 60)), int(r.integers(1 << 30)))))

    threads = [threading.Thread(target=noise, args=(s,)) for s in range(3)]
    for t in threads:
        t.start()
    cl = server.submit_cluster(lib[64][:150], 2.5, 4)
    for k, x in enumerate(probes):
        tickets[k] = server.submit(x)
    for t in threads:
        t.join()
    mixed = [server.wait(tickets[k]) for k in range(len(probes))]
    for t in others:
        server.wait(t)
    server.wait_cluster(cl)
    for (ia, va), (ib, vb) in zip(alone, mixed):
        np.testing.assert_array_equal(ia, ib)
        np.testing.assert_array_equal(va, vb)
    st = server.stats()
    assert st["batches"] >= 1 and st["queries_done"] >= 3 and st["p99_ms"] >= st["p50_ms"] > 0


def test_cluster_job_matches_engine_optics(server, library, engine):
    lib, _, _ = library
    x = lib[128][:90]
    labels = server.wait_cluster(server.submit_cluster(x, 3.0, 5))
    m = engine.all_vs_all(x, CrmsdOptions(out_type="f32"))
    _, _, want = K.optics(m, 3.0, 5)
    np.testing.assert_array_equal(labels, want)


def test_plain_precision_server(library, oracle_mod, enginelib):
    from bioshell_gb300 import CrmsdServer
    lib, _, _ = library
    s = CrmsdServer({64: lib[64]}, top_k=TOPK, precision="plain64")
    try:
        x = _queries(library, 64, 4, 21)
        idx, val = s.wait(s.submit(x))
        _check_against_oracle(lib[64], x, idx, val, oracle_mod)
    finally:
        s.close()


def test_out_of_range_query_uses_the_fp64_path(server, library, oracle_mod):
    lib, _, _ = library
    x = _queries(library, 64, 2, 31) * 40.0  # far beyond the bucket's grid range
    before = server.stats()["plain_fallbacks"]
    idx, val = server.wait(server.submit(x))
    assert server.stats()["plain_fallbacks"] == before + 1
    _check_against_oracle(lib[64], x, idx, val, oracle_mod)


def test_server_errors(server, library):
    with pytest.raises(CrmsdError) as e:
        server.submit(np.zeros((2, 77, 3)))  # no bucket of that length
    assert e.value.status == 1
    x = _queries(library, 64, 3, 41)
    x[1, 5, 2] = np.nan
    t = server.submit(x)
    with pytest.raises(CrmsdError) as e:
        server.wait(t)
    assert e.value.status == 6
    idx, _ = server.wait(server.submit(_queries(library, 64, 2, 42)))  # still serving
    assert np.all(idx >= 0)


def test_library_index_keeps_results(oracle_mod, enginelib):
    """A library index prunes the screen but changes no result: an indexed
    server and an unindexed one return the same indices and values, bit for
    bit, for single-family and mixed-family requests and with exact
    duplicates in the library (ties broken by library index)."""
    from bioshell_gb300 import CrmsdServer
    rng = np.random.default_rng(91)
    parts = [synth.decoys(synth.base_chain(64, rng), 480, rng, sigma=(0.3, 3.0)) for _ in range(8)]
    lib = np.concatenate(parts)
    lib = np.concatenate([lib, lib[rng.choice(len(lib), 96, replace=False)]])  # exact duplicates
    plain = CrmsdServer({64: lib}, top_k=TOPK, max_inflight=2, index_min=-1)
    indexed = CrmsdServer({64: lib}, top_k=TOPK, max_inflight=2, index_min=1)
    try:
        reqs = []
        for f, q in ((0, 45), (3, 1), (5, 120)):
            base = parts[f][0] - parts[f][0].mean(axis=0)
            reqs.append(synth.decoys(base, q, rng, sigma=(0.3, 2.0)))
        # one request mixing families, and library members themselves (ties)
        reqs.append(np.concatenate([synth.decoys(p[0] - p[0].mean(axis=0), 7, rng, sigma=(0.3, 2.0))
                                    for p in parts]))
        reqs.append(lib[rng.choice(len(lib), 30, replace=False)])
        for x in reqs:
            a = plain.wait(plain.submit(x))
            b = indexed.wait(indexed.submit(x))
            np.testing.assert_array_equal(a[0], b[0])
            np.testing.assert_array_equal(a[1], b[1])
        _check_against_oracle(lib, reqs[3][:4], *[v[:4] for v in indexed.wait(indexed.submit(reqs[3]))],
                              oracle_mod)
        st = indexed.stats()
        assert 0 < st["pairs_screened"]
    finally:
        plain.close()
        indexed.close()


def test_trace_records_batches_and_requests(library, enginelib, tmp_path, monkeypatch):
    """BS_SERVER_TRACE: one B line per batch and one R line per request, written
    when the server is destroyed; results are the same as without the trace."""
    from bioshell_gb300 import CrmsdServer
    lib, _, _ = library
    path = tmp_path / "trace.csv"
    x = _queries(library, 64, 5, 9)
    plain = CrmsdServer(lib, top_k=TOPK, max_inflight=2)
    want = plain.wait(plain.submit(x))
    plain.close()
    monkeypatch.setenv("BS_SERVER_TRACE", str(path))
    s = CrmsdServer(lib, top_k=TOPK, max_inflight=2)
    monkeypatch.delenv("BS_SERVER_TRACE")
    tickets = [s.submit(x), s.submit(_queries(library, 128, 3, 10))]
    got = s.wait(tickets[0])
    s.wait(tickets[1])
    s.close()
    assert np.array_equal(got[0], want[0]) and np.array_equal(got[1], want[1])
    lines = path.read_text().splitlines()
    assert lines[0] == "# server"
    b = [ln.split(",") for ln in lines if ln.startswith("B,")]
    r = [ln.split(",") for ln in lines if ln.startswith("R,")]
    assert len(r) == 2 and {int(f[4]) for f in r} == {5, 3}
    assert len(b) >= 1 and sum(int(f[5]) for f in b) == 8
    for f in r:  # submitted before completed, carried by a traced batch, status OK
        assert float(f[5]) <= float(f[6]) and int(f[8]) == 0
        assert int(f[7]) in {int(g[2]) for g in b}


def test_top50_of_a_20000_library_against_oracle(oracle_mod, enginelib):
    """Top-50 over a 20,000-structure bucket (large enough for the library
    index: the head-set pre-screen and the pruned screen both run) for 300
    queries: every returned value within 1e-4 A of the FP64 oracle, and every
    member of the oracle's top 50 that lies more than 2e-4 A inside the cut
    returned.  A screen bracket that missed its pair's true crmsd would drop
    such a member."""
    from bioshell_gb300 import CrmsdServer
    rng = np.random.default_rng(31)
    lib, fams = _family_library(rng, 64, 20000, families=8)
    srv = CrmsdServer({64: lib}, top_k=50, max_inflight=2)
    try:
        qs = []
        for k in range(300):
            base = fams[k % 8][0]
            qs.append(synth.decoys(base - base.mean(axis=0), 1, rng, sigma=(0.3, 2.5))[0])
        x = np.stack(qs)
        tickets = [srv.submit(x[o:o + 30]) for o in range(0, 300, 30)]
        res = [srv.wait(t) for t in tickets]
        idx = np.concatenate([r[0] for r in res])
        val = np.concatenate([r[1] for r in res])
    finally:
        srv.close()
    n = lib.shape[0]
    both = np.concatenate([x, lib])
    ii = np.repeat(np.arange(300), n)
    jj = np.tile(np.arange(300, 300 + n), 300)
    ref = oracle_mod.crmsd_pairs(both, ii, jj).reshape(300, n)
    missing = 0
    for r in range(300):
        np.testing.assert_allclose(val[r], ref[r, idx[r]], rtol=0, atol=TOL)
        order = np.lexsort((np.arange(n), ref[r]))
        kth = ref[r, order[49]]
        want = set(order[:50][ref[r, order[:50]] < kth - 2 * TOL].tolist())
        missing += len(want - set(idx[r].tolist()))
        assert np.all(np.diff(val[r]) >= 0)
    assert missing == 0
