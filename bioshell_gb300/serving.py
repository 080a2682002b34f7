"""Serving handle over a device-resident structure library (``bs_server_*``
in ``include/bioshell_crmsd.h``): the ``CrmsdServer::{new, submit, wait}``
API a maintainer would add beside ``crmsd_all_vs_all``.

``CrmsdServer({L: coords})`` copies the library (one ``[n][L][3]`` array per
chain length) to the GPU once.  ``submit(query)`` queues ``q`` structures of
one of those lengths and returns a ticket; ``wait(ticket)`` returns, for each
query structure, the ``top_k`` nearest library structures of that length by
crmsd: ``(indices[q][k], rmsd[q][k])``, ascending.  ``submit_cluster`` queues
an all-vs-all + OPTICS job (bioshell-clustering/src/optics.rs:51-148) over its
own structures.  Requests are batched continuously on the GPU by the
library's scheduler thread; ``stats()`` reports latency percentiles and
pairs/s.
"""
from __future__ import annotations

import ctypes
from typing import Dict, Optional

import numpy as np

from . import lib as _l


class CrmsdServer:
    def __init__(self, library: Dict[int, np.ndarray], device: int = 0, top_k: int = 50, max_inflight: int = 4,
                 hbm_budget: int = 0, precision: str = "mixed", max_batch_rows: int = 0,
                 tolerance: Optional[float] = None, index_min: int = 0):
        self._lib = _l.load()
        self.top_k = int(top_k)
        lengths = sorted(library)
        self._keep = [np.ascontiguousarray(library[L], dtype=np.float64) for L in lengths]
        for L, x in zip(lengths, self._keep):
            if x.ndim != 3 or x.shape[1] != L or x.shape[2] != 3:
                raise ValueError(f"library bucket {L} must be [n][{L}][3]")
        nb = len(lengths)
        Ls = (ctypes.c_int32 * nb)(*lengths)
        ns = (ctypes.c_int64 * nb)(*[x.shape[0] for x in self._keep])
        ptrs = (ctypes.c_void_p * nb)(*[x.ctypes.data for x in self._keep])
        cfg = _l.bs_server_config()
        cfg.nbuckets = nb
        cfg.bucket_L = Ls
        cfg.bucket_n = ns
        cfg.bucket_xyz = ptrs
        cfg.top_k = self.top_k
        cfg.max_inflight = int(max_inflight)
        cfg.hbm_budget = int(hbm_budget)
        cfg.precision = _l.PRECISION[precision]
        cfg.max_batch_rows = int(max_batch_rows)
        cfg.tolerance = float(tolerance or 0.0)
        cfg.index_min = int(index_min)  # buckets this large get a library index (0: 16384, < 0: never)
        h = ctypes.c_void_p()
        st = self._lib.bs_server_create(ctypes.byref(h), int(device), ctypes.byref(cfg))
        if st != _l.BS_OK:
            raise _l.CrmsdError(st, "bs_server_create")
        self._h = h
        self._keep = None  # the library now lives on the device
        self.lengths = lengths
        self._shapes = {}

    def close(self):
        if self._h:
            self._lib.bs_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st: int):
        if st != _l.BS_OK:
            raise _l.CrmsdError(st, self._lib.bs_server_last_error(self._h).decode())

    def submit(self, query) -> int:
        x = np.ascontiguousarray(query, dtype=np.float64)
        if x.ndim == 2:
            x = x[None]
        t = ctypes.c_int64()
        self._check(self._lib.bs_server_submit(self._h, x.ctypes.data, x.shape[0], x.shape[1], ctypes.byref(t)))
        self._shapes[t.value] = x.shape[0]
        return t.value

    def submit_cluster(self, xyz, eps: float, min_points: int) -> int:
        x = np.ascontiguousarray(xyz, dtype=np.float64)
        t = ctypes.c_int64()
        self._check(self._lib.bs_server_submit_cluster(self._h, x.ctypes.data, x.shape[0], x.shape[1], float(eps),
                                                       int(min_points), ctypes.byref(t)))
        self._shapes[t.value] = x.shape[0]
        return t.value

    def poll(self, ticket: int) -> bool:
        d = ctypes.c_int32()
        self._check(self._lib.bs_server_poll(self._h, int(ticket), ctypes.byref(d)))
        return bool(d.value)

    def wait(self, ticket: int, timeout: float = 0.0):
        q = self._shapes.pop(ticket)
        idx = np.empty((q, self.top_k), dtype=np.int64)
        val = np.empty((q, self.top_k), dtype=np.float64)
        self._check(self._lib.bs_server_wait(self._h, int(ticket), idx.ctypes.data, val.ctypes.data, float(timeout)))
        return idx, val

    def wait_cluster(self, ticket: int, timeout: float = 0.0) -> np.ndarray:
        n = self._shapes.pop(ticket)
        cl = np.empty(n, dtype=np.int64)
        self._check(self._lib.bs_server_wait_cluster(self._h, int(ticket), cl.ctypes.data, float(timeout)))
        return cl

    def cancel(self, ticket: int) -> bool:
        """Cancels a request still in the queue (True); one already on the GPU
        or done runs to completion (False).  A cancelled request's wait raises
        CrmsdError with status BS_ERR_CANCELLED."""
        c = ctypes.c_int32()
        self._check(self._lib.bs_server_cancel(self._h, int(ticket), ctypes.byref(c)))
        return bool(c.value)

    def stats(self) -> dict:
        s = _l.bs_server_stats()
        self._check(self._lib.bs_server_get_stats(self._h, ctypes.byref(s)))
        return s.as_dict()

    def reset_stats(self):
        self._check(self._lib.bs_server_reset_stats(self._h))


# ---- the server's timing trace (BS_SERVER_TRACE) ---------------------------
_B_FIELDS = ("slot", "batch", "kind", "bucket", "rows", "nreq", "hand_ms", "launch_begin_ms", "launch_end_ms",
             "event_ms", "finish_ms", "dev_grows", "host_grows", "grow_ms")
_R_FIELDS = ("id", "kind", "bucket", "q", "submit_ms", "done_ms", "batch", "status")


def read_trace(path: str):
    """Parse a trace written by a server created with ``BS_SERVER_TRACE=path``.

    Returns one dict per server in the file (servers of one process append),
    each with ``segments``: the records between ``reset_stats`` calls (times
    count from the latest reset), each a dict of ``batches`` and
    ``requests`` (lists of dicts keyed by the trace's field names).
    """
    servers = []
    with open(path) as fh:
        for line in fh:
            line = line.strip()
            if line == "# server":
                servers.append({"segments": [{"batches": [], "requests": []}]})
            elif line == "# reset" and servers:
                servers[-1]["segments"].append({"batches": [], "requests": []})
            elif line[:2] in ("B,", "R,") and servers:
                parts = line.split(",")[1:]
                names = _B_FIELDS if line[0] == "B" else _R_FIELDS
                rec = {k: (float(v) if k.endswith("_ms") else int(v)) for k, v in zip(names, parts)}
                servers[-1]["segments"][-1]["batches" if line[0] == "B" else "requests"].append(rec)
    return servers


def slow_requests(segment: dict, percentile: float = 99.0):
    """The query requests of one trace segment at or above the given latency
    percentile, each with where its time went: ``wait`` (submit to hand-off
    to a slot), ``launch`` (host work of the batch launch), ``device`` (until
    the batch's work completed), ``finish`` (results to the requests)."""
    import numpy as np
    batches = {b["batch"]: b for b in segment["batches"]}
    reqs = [r for r in segment["requests"] if r["kind"] == 0 and r["status"] == 0]
    if not reqs:
        return []
    lat = np.array([r["done_ms"] - r["submit_ms"] for r in reqs])
    cut = float(np.percentile(lat, percentile))
    out = []
    for r, ms in zip(reqs, lat):
        b = batches.get(r["batch"])
        if ms < cut or b is None:
            continue
        out.append({"id": r["id"], "latency_ms": float(ms), "rows": b["rows"], "slot": b["slot"],
                    "wait": b["hand_ms"] - r["submit_ms"], "launch": b["launch_end_ms"] - b["launch_begin_ms"],
                    "device": b["event_ms"] - b["launch_end_ms"], "finish": b["finish_ms"] - b["event_ms"],
                    "grows": b["dev_grows"] + b["host_grows"]})
    return sorted(out, key=lambda d: -d["latency_ms"])
