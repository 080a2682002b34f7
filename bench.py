#!/usr/bin/env python
"""Benchmark of the GB300 crmsd engine: all-vs-all crmsd pairs/s.

Workload (default): 50,000 synthetic decoys x 300 CA atoms, 5% near-duplicates
(noise sigma 0.01 A), every one of the 1,249,975,000 pairs per step, mixed
precision (exact bf16 digit products on tcgen05 tensor cores + FP32/integer
QCP epilogue), f64 packed-triangle output.

One JSON line on stdout (rank 0):
  value     pairs/s with coordinates and result resident in HBM, CUDA events
            on the engine's stream around K steps;
  e2e       the same through the C ABI with pinned HOST buffers: every step
            copies the coordinates in and the whole f64 triangle out;
  roofline  the tensor-core kernel: algorithmic 18*L flops/pair over its
            event-timed duration, against the measured bf16 peak;
  streaming_roofline  the preparation pass: 48 L + 40 bytes per structure
            over its event-timed duration, against the measured HBM rate;
  plain64   the plain FP64 GPU path on the same workload (the denominator);
  serving   a device-resident library of 200,000 decoys bucketed by chain
            length (L 64/128/256/512 at 85/9/4/2%); queries arrive as a
            Poisson process at 2,000 req/s, each q ~ U{1..512} structures of
            a bucket drawn by library share, answered with the top-50
            nearest by crmsd; 500-5,000-decoy clustering jobs are mixed in.
            p50/p99 latency (submit -> results), pairs/s, and the capacity
            of the mixed and plain FP64 servers (closed loop);
  batched   256 decoy sets (N log-uniform in [50, 4000], L log-uniform in
            [40, 800], sigma U[0.2, 6]) in one graph-replayed launch per
            step, against the plain FP64 path on the same sets, with per-set
            OPTICS partitions compared (eps 3 A, min_points 5);
  accuracy  |dRMSD| vs the FP64 oracle on 1e6 seeded pairs + all
            near-duplicate pairs;
  cpu_baseline  the oracle on this host's cores on a bounded sample.
``--impl reference`` times the CPU oracle alone (the reference has no crmsd
implementation of its own; see the oracle's header).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from bioshell_gb300 import synth  # noqa: E402

METRIC = "crmsd pairs/s (all-vs-all, mixed precision)"
UNIT = "pairs/s"


def whole_job_rate(ms, units_per_rank, steps, world, dist=None, device="cuda"):
    """The slowest rank's time over `steps` steps (max over ranks) and the
    whole job's rate: each of the `world` ranks processes `units_per_rank`
    units per step (weak scaling: independent replicas or disjoint row
    ranges, no exchange between ranks)."""
    if dist is not None and world > 1:
        import torch
        t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    return ms, world * units_per_rank * steps / (ms * 1e-3)


def args_():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--n", type=int, default=None, help="override the number of decoys (debug only)")
    p.add_argument("--L", type=int, default=None, help="override the chain length (debug only)")
    p.add_argument("--skip-plain", action="store_true")
    p.add_argument("--skip-accuracy", action="store_true")
    p.add_argument("--skip-batched", action="store_true")
    p.add_argument("--skip-serving", action="store_true")
    p.add_argument("--serve-seconds", type=float, default=3.0)
    p.add_argument("--serve-rate", type=float, default=2000.0)
    p.add_argument("--serve-inflight", type=int, default=4, help="device slots of the serving benchmark")
    p.add_argument("--cpu-seconds", type=float, default=10.0)
    p.add_argument("--probe-serving", type=int, default=0, metavar="K",
                   help="only run K query batches of 256 structures of the 64-atom bucket through a one-slot "
                        "server over the 200,000-structure library (a profiling target), print one JSON line")
    return p.parse_args()


def workload(a):
    w = synth.MIXED_50K
    if a.n or a.L:
        w = synth.Workload(f"decoys-{a.n or w.n}x{a.L or w.L}-neardup5", n=a.n or w.n, L=a.L or w.L,
                           near_dup_frac=w.near_dup_frac, near_dup_sigma=w.near_dup_sigma, seed=w.seed)
    return w


def tri_pairs(n, t):
    t = np.asarray(t, dtype=np.int64)
    i = np.floor((2 * n - 1 - np.sqrt((2 * n - 1) ** 2 - 8 * t.astype(np.float64))) / 2).astype(np.int64)
    i = np.where(i * n - i * (i + 1) // 2 > t, i - 1, i)
    i = np.where((i + 1) * n - (i + 1) * (i + 2) // 2 <= t, i + 1, i)
    j = t - (i * n - i * (i + 1) // 2) + i + 1
    return i, j


def issued_flops(n, L):
    """Tensor-core flops the mixed kernel issues per call: every tile of 40 x
    20 structures (128 x 64 rows) holding a pair i < j (column block J >= 2I)
    runs 9 digit products over the 16-padded chain length."""
    nba, nbb = (n + 39) // 40, (n + 19) // 20
    tiles = sum(max(0, nbb - 2 * i) for i in range(nba))
    lp = ((L + 15) // 16) * 16
    return tiles * 2.0 * 128 * 64 * lp * 9


def host_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def cpu_baseline(x, seconds, seed=99):
    """The FP64 oracle on this host's cores, on a bounded random sample."""
    from oracle import oracle
    oracle.build()
    n = x.shape[0]
    rng = np.random.default_rng(seed)
    threads = host_threads()
    npairs = n * (n - 1) // 2
    # the sample's size from a probe that runs long enough to time: a first
    # call (thread start-up, first touch of the coordinates) is not counted,
    # then the probe grows tenfold until it takes at least 0.2 s
    probe = min(npairs, 20000)
    t = rng.choice(npairs, probe, replace=False)
    i, j = tri_pairs(n, t)
    oracle.crmsd_pairs(x, i, j, nthreads=threads)
    while True:
        t = rng.choice(npairs, probe, replace=False)
        i, j = tri_pairs(n, t)
        t0 = time.perf_counter()
        oracle.crmsd_pairs(x, i, j, nthreads=threads)
        dt = time.perf_counter() - t0
        if dt >= 0.2 or probe >= npairs or dt * 10 >= seconds:
            break
        probe = min(npairs, probe * 10)
    size = int(min(npairs, max(probe, probe * seconds / max(dt, 1e-6))))
    t = rng.choice(npairs, size, replace=False) if size < npairs else np.arange(npairs)
    i, j = tri_pairs(n, t)
    t0 = time.perf_counter()
    oracle.crmsd_pairs(x, i, j, nthreads=threads)
    dt = time.perf_counter() - t0
    return {"value": size / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{size} seeded random pairs of the same {n}x{x.shape[1]} set, {dt:.1f} s"}


class Clocks:
    """nvidia-smi samples during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.f = None

    def __enter__(self):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", str(self.device)], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            self.proc.wait()
        self.f.flush()

    def summary(self):
        rows = []
        with open(self.f.name) as fh:
            for line in fh:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.f.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}

        def num(v):
            try:
                return float(v)
            except ValueError:
                return None

        sm = [num(r[1]) for r in rows if num(r[1])]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for k, nm in enumerate(names):
                if r[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": num(rows[0][2]),
                "reasons": sorted(reasons), "samples": len(rows),
                "power_w_max": max((num(r[3]) or 0.0) for r in rows)}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            p = json.load(fh)
        return p, "measured"
    except OSError:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


def fp64_peak(device):
    """The GPU's FP64 FMA rate in FLOP/s, measured in-tree (bs_diag_fp64_peak)."""
    import ctypes
    from bioshell_gb300 import lib as _l
    v = ctypes.c_double()
    st = _l.load().bs_diag_fp64_peak(int(device), ctypes.byref(v))
    return v.value if st == 0 else None


def profiled_traffic(name):
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as fh:
            return json.load(fh).get(name)
    except (OSError, ValueError):
        return None


def run_neighbors(eng, xd, outd, n, torch, eps=1.0, steps=3):
    """eps-neighbour lists of the headline set without the dense matrix: device
    time of the sparse form, and a check of sampled rows against the dense
    result of the same set."""
    rp, col, dist = eng.neighbors(xd, eps)
    ms = []
    for _ in range(steps):
        rp, col, dist = eng.neighbors(xd, eps)
        ms.append(eng.metrics()["ms_total"])
    ok = True
    rows = (0, 1, n // 2, n - 1)
    for i in rows:
        j = np.arange(n)
        j = j[j != i]
        lo, hi = np.minimum(i, j), np.maximum(i, j)
        t = lo * n - lo * (lo + 1) // 2 + (hi - lo - 1)
        d = outd[torch.from_numpy(t).cuda()].cpu().numpy().astype(np.float32)
        keep = d <= eps
        o = np.lexsort((j[keep], d[keep]))
        ok &= bool(np.array_equal(col[rp[i]:rp[i + 1]], j[keep][o]) and
                   np.array_equal(dist[rp[i]:rp[i + 1]], d[keep][o]))
    nnz = int(rp[-1])
    msd = statistics.median(ms)
    return {"eps": eps, "nnz": nnz, "mean_neighbors": nnz / n, "ms_device": msd,
            "pairs_per_s": n * (n - 1) / 2 / (msd * 1e-3), "csr_bytes": int(8 * (n + 1) + 8 * nnz),
            "dense_f32_bytes": int(4 * n * (n - 1) // 2), "rows_checked_against_dense": len(rows), "match": ok}


def run_superpose(eng, xd, x, torch, npairs=1_000_000, steps=3):
    """Rototranslations of random pairs of the headline set (device-resident
    coordinates, pair lists and outputs): device time, and a sample checked
    against the host copy of the same math."""
    import ctypes
    n, L = x.shape[0], x.shape[1]
    rng = np.random.default_rng(31)
    ii = torch.from_numpy(rng.integers(0, n, npairs)).cuda()
    jj = torch.from_numpy(rng.integers(0, n, npairs)).cuda()
    out = (torch.empty((npairs, 3, 3), dtype=torch.float64, device="cuda"),
           torch.empty((npairs, 3), dtype=torch.float64, device="cuda"),
           torch.empty(npairs, dtype=torch.float64, device="cuda"))
    eng.superpose_pairs(xd, ii, jj, out)
    ms = []
    for _ in range(steps):
        eng.superpose_pairs(xd, ii, jj, out)
        ms.append(eng.metrics()["ms_main"])
    sel = rng.choice(npairs, 64, replace=False)
    rot = out[0][torch.from_numpy(sel).cuda()].cpu().numpy()
    rm = out[2][torch.from_numpy(sel).cuda()].cpu().numpy()
    si, sj = ii.cpu().numpy()[sel], jj.cpu().numpy()[sel]
    worst_r = worst_m = 0.0
    for t in range(len(sel)):
        hr, ht, hm = np.empty(9), np.empty(3), ctypes.c_double()
        a, b = np.ascontiguousarray(x[si[t]]), np.ascontiguousarray(x[sj[t]])
        eng._lib.bs_selftest_superpose(a.ctypes.data, b.ctypes.data, L, hr.ctypes.data, ht.ctypes.data,
                                       ctypes.byref(hm))
        worst_r = max(worst_r, float(np.abs(rot[t] - hr.reshape(3, 3)).max()))
        worst_m = max(worst_m, abs(float(rm[t]) - hm.value))
    msd = statistics.median(ms)
    return {"pairs": npairs, "L": L, "ms_device": msd, "pairs_per_s": npairs / (msd * 1e-3),
            "sample_checked": len(sel), "max_abs_rot_vs_host": worst_r, "max_abs_rmsd_vs_host": worst_m}


def run_formats(eng, torch, n_models=1000, L=300, n_tsv=4000):
    """Throughput of the formats either side of the path: multi-model PDB
    ingestion (a synthetic ensemble of n_models x L residues, 4 atoms each,
    CA selected) and TSV export of a device-resident f64 triangle."""
    import tempfile
    import time
    from bioshell_gb300 import formats as F
    rng = np.random.default_rng(12)
    base = synth.base_chain(L, rng)
    ens = synth.decoys(base, n_models, rng)
    names = (" N  ", " CA ", " C  ", " O  ")
    with tempfile.TemporaryDirectory() as d:
        pdb = os.path.join(d, "ens.pdb")
        with open(pdb, "w") as fh:
            for m in range(n_models):
                fh.write(f"MODEL     {m + 1:4d}\n")
                rows = []
                for r in range(L):
                    for k, nm in enumerate(names):
                        x, y, z = ens[m, r] + 0.5 * k
                        rows.append(f"ATOM  {4 * r + k + 1:5d} {nm} ALA A{r + 1:4d}    {x:8.3f}{y:8.3f}{z:8.3f}"
                                    f"  1.00  0.00           {nm.strip()[0]}\n")
                fh.write("".join(rows))
                fh.write("ENDMDL\n")
        size = os.path.getsize(pdb)
        t0 = time.perf_counter()
        ca = F.read_models(pdb, ca_only=True)
        t_read = time.perf_counter() - t0
        # the CA record of residue r is written at ens + 0.5 (atom index 1)
        want = np.array([float(f"{v:.3f}") for v in (ens[:4] + 0.5).ravel()]).reshape(4, L, 3)
        ok = bool(np.array_equal(ca[:4], want) and ca.shape == (n_models, L, 3))
        x = synth.decoys(synth.base_chain(150, rng), n_tsv, rng)
        npair = n_tsv * (n_tsv - 1) // 2
        dev = torch.empty(npair, dtype=torch.float64, device="cuda")
        eng.all_vs_all(torch.from_numpy(x).cuda(), out=dev)
        tsv = os.path.join(d, "m.tsv")
        labels = [f"model_{i}" for i in range(n_tsv)]
        t0 = time.perf_counter()
        F.write_tsv(tsv, dev, labels, n=n_tsv)
        t_tsv = time.perf_counter() - t0
        tsv_bytes = os.path.getsize(tsv)
    return {"models": {"file": f"PDB, {n_models} models x {L} residues x 4 atoms, CA selected",
                       "bytes": size, "seconds": t_read, "MB_per_s": size / t_read / 1e6,
                       "models_per_s": n_models / t_read, "exact": ok},
            "tsv_export": {"pairs": npair, "source": "device f64 triangle", "bytes": tsv_bytes, "seconds": t_tsv,
                           "lines_per_s": npair / t_tsv, "MB_per_s": tsv_bytes / t_tsv / 1e6,
                           "threads": host_threads()}}


def run_hierarchical(eng, n=3000, L=150, rule="average"):
    """Agglomerative clustering of an n-structure crmsd matrix: the host
    version against the GPU one (same merges required)."""
    import time
    from bioshell_gb300 import clustering as K
    from bioshell_gb300.crmsd import CrmsdOptions
    rng = np.random.default_rng(13)
    x = synth.decoys(synth.base_chain(L, rng), n, rng)
    m = eng.all_vs_all(x, CrmsdOptions(out_type="f32"))
    t0 = time.perf_counter()
    dev = K.hierarchical_clustering(m, rule, engine=eng)
    t_gpu = time.perf_counter() - t0
    kernel_ms = eng.metrics()["ms_main"]
    t0 = time.perf_counter()
    host = K.hierarchical_clustering(m, rule)
    t_host = time.perf_counter() - t0
    same = bool(np.array_equal(dev.merges, host.merges) and np.array_equal(dev.dist, host.dist))
    return {"n": n, "rule": rule, "gpu_s": t_gpu, "gpu_kernel_ms": kernel_ms,
            "host_s": t_host, "speedup": t_host / t_gpu, "identical_merges": same}


def run_batched(a, eng, stream, torch):
    """The batched form: all sets in one call per step (graph replay)."""
    from bioshell_gb300 import clustering as K
    from bioshell_gb300.crmsd import CrmsdMatrix, CrmsdOptions
    sets = synth.batched_sets()
    ns = [x.shape[0] for x in sets]
    pairs = sum(n * (n - 1) // 2 for n in ns)
    dev = [torch.from_numpy(x).cuda() for x in sets]
    outs = [torch.empty(n * (n - 1) // 2, dtype=torch.float64, device="cuda") for n in ns]
    tuned = 0
    t_tune = time.perf_counter()
    opts = CrmsdOptions(autotune=True)
    for _ in range(a.warmup):  # the first call times the tile shapes of every set class
        eng.batched(dev, opts, outs=outs)
        tuned += eng.metrics()["tuned_classes"]
    t_tune = time.perf_counter() - t_tune
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    mets = []
    ev0.record(stream)
    for _ in range(a.steps):
        eng.batched(dev, opts, outs=outs)
        mets.append(eng.metrics())
    ev1.record(stream)
    ev1.synchronize()
    ms = ev0.elapsed_time(ev1) / a.steps
    graph = mets[-1]["graph"]
    # the fixed default (every set on 40 x 20 tiles) against the tuned shapes
    wide = CrmsdOptions()
    eng.batched(dev, wide, outs=outs)
    torch.cuda.synchronize()
    ev0.record(stream)
    for _ in range(a.steps):
        eng.batched(dev, wide, outs=outs)
    ev1.record(stream)
    ev1.synchronize()
    ms_wide = ev0.elapsed_time(ev1) / a.steps
    tuning = eng.tuning()
    n_narrow_classes = sum(1 for c in tuning["classes"] if c[2] == "narrow")
    # plain FP64 path on the same sets
    outs64 = [torch.empty_like(o) for o in outs]
    eng.batched(dev, CrmsdOptions(precision="plain64"), outs=outs64)
    m64 = eng.metrics()
    gap = max(float((o - p).abs().max()) if o.numel() else 0.0 for o, p in zip(outs, outs64))
    # per-set OPTICS partitions, mixed vs FP64
    eps, min_points = 3.0, 5
    same = 0
    near_eps = 0
    for n, o, p in zip(ns, outs, outs64):
        mo, mp = o.cpu().numpy(), p.cpu().numpy()
        _, _, co = K.optics(CrmsdMatrix(n, mo), eps, min_points)
        _, _, cp = K.optics(CrmsdMatrix(n, mp), eps, min_points)
        same += bool(np.array_equal(co, cp))
        near_eps += bool(np.any(np.abs(mp - eps) <= gap))
    # end to end: pinned host buffers in and out
    hin = []
    for x in sets:
        h = eng.host_empty(x.shape, np.float64)
        h[...] = x
        hin.append(h)
    hout = [eng.host_empty((n * (n - 1) // 2,), np.float64) for n in ns]
    eng.batched(hin, opts, outs=hout)
    t_e = []
    for _ in range(max(1, min(a.steps, 2))):
        eng.batched(hin, opts, outs=hout)
        t_e.append(eng.metrics()["ms_total"])
    ms_e2e = statistics.mean(t_e)
    Ls = [x.shape[1] for x in sets]
    return {"workload": "256 decoy sets, N logU[50,4000], L logU[40,800], sigma U[0.2,6], seed 3",
            "sets": len(sets), "structures": int(sum(ns)), "pairs": int(pairs), "L_max": int(max(Ls)),
            "value": pairs / (ms * 1e-3), "unit": UNIT, "ms_per_step": ms, "graph": graph,
            "ms_prep": statistics.mean(m["ms_prep"] for m in mets),
            "ms_main": statistics.mean(m["ms_main"] for m in mets),
            "ms_refine": statistics.mean(m["ms_refine"] for m in mets),
            "pairs_refined": int(mets[-1]["pairs_refined"]),
            "autotune": {"classes_timed": tuned, "narrow_sets": int(mets[-1]["narrow_jobs"]),
                         "classes_narrow": n_narrow_classes, "classes_wide": len(tuning["classes"]) - n_narrow_classes,
                         "ms_all_wide_default": ms_wide, "gain_vs_all_wide": ms_wide / ms,
                         "warmup_s_incl_tuning": t_tune},
            "e2e": {"value": pairs / (ms_e2e * 1e-3), "unit": UNIT, "ms_per_step": ms_e2e,
                    "h2d_bytes_per_step": int(sum(x.nbytes for x in sets)), "d2h_bytes_per_step": int(pairs * 8)},
            "plain64": {"value": pairs / (m64["ms_total"] * 1e-3), "unit": UNIT, "ms_per_step": m64["ms_total"]},
            "speedup_vs_plain64": m64["ms_total"] / ms,
            "max_abs_vs_plain64": gap,
            "optics": {"eps": eps, "min_points": min_points, "identical_labels": same, "sets": len(sets),
                       "sets_with_distance_within_gap_of_eps": near_eps}}


def _closed_loop(srv, pools, shares, seconds, rng, max_inflight=8):
    """Back-to-back queries for `seconds`: the server's throughput ceiling."""
    import collections
    srv.reset_stats()
    Ls = [L for L, _ in shares]
    ps = np.array([p for _, p in shares])
    q = collections.deque()
    t_end = time.perf_counter() + seconds
    while time.perf_counter() < t_end:
        while len(q) < max_inflight:
            L = int(rng.choice(Ls, p=ps / ps.sum()))
            n = int(rng.integers(1, 513))
            o = int(rng.integers(0, pools[L].shape[0] - n + 1))
            q.append(srv.submit(pools[L][o:o + n]))
        srv.wait(q.popleft())
    while q:
        srv.wait(q.popleft())
    return srv.stats()


def _open_loop(srv, pools, shares, rate, T, rng, q_fixed=None, cjobs=()):
    """Poisson arrivals at `rate` for `T` seconds: queries of q ~ U{1..512}
    structures (or exactly q_fixed) of a bucket drawn by library share, with
    the clustering jobs spread over the run.  Returns the server's stats for
    the run, the submit lags (ms), the submitting time and the request count."""
    import queue as qmod
    import threading
    srv.reset_stats()
    gaps = rng.exponential(1.0 / rate, size=int(rate * T * 1.5) + 10)
    times = np.cumsum(gaps)
    times = times[times < T]
    Ls = np.array([L for L, _ in shares])
    ps = np.array([p for _, p in shares])
    bk = rng.choice(Ls, size=len(times), p=ps / ps.sum())
    qs = np.full(len(times), q_fixed) if q_fixed else rng.integers(1, 513, size=len(times))
    offs = [int(rng.integers(0, pools[int(L)].shape[0] - int(n) + 1)) for L, n in zip(bk, qs)]
    ctimes = np.linspace(0.1, T * 0.9, len(cjobs))
    tickets = qmod.Queue()

    def collect():
        while True:
            item = tickets.get()
            if item is None:
                return
            kind, t = item
            if kind == 0:
                srv.wait(t)
            else:
                srv.wait_cluster(t)

    th = threading.Thread(target=collect)
    th.start()
    lag = []
    ci = 0
    start = time.perf_counter()
    for k, t_arr in enumerate(times):
        while ci < len(cjobs) and ctimes[ci] <= t_arr:
            tickets.put((1, srv.submit_cluster(cjobs[ci], 3.0, 5)))
            ci += 1
        now = time.perf_counter() - start
        if t_arr > now:
            time.sleep(t_arr - now)
        lag.append((time.perf_counter() - start - t_arr) * 1e3)
        L, n, o = int(bk[k]), int(qs[k]), offs[k]
        tickets.put((0, srv.submit(pools[L][o:o + n])))
    submit_s = time.perf_counter() - start
    tickets.put(None)
    th.join()
    return srv.stats(), lag, submit_s, int(len(times))


def run_serving(a):
    """Open-loop Poisson load against the resident library, then capacity."""
    from bioshell_gb300 import CrmsdServer
    lib, bases = synth.serving_library()
    pools = synth.serving_queries(bases)
    shares = list(synth.SERVING_BUCKETS)
    rng = np.random.default_rng(6)
    # clustering jobs mixed in: all-vs-all + OPTICS of 500-5000 decoys
    cjobs = []
    for k in range(4):
        L = 64 if k % 2 == 0 else 128
        n = int(rng.integers(500, 5001))
        cjobs.append(synth.decoys(bases[L][k], n, rng, (0.3, 4.0)))
    t0 = time.perf_counter()
    srv = CrmsdServer(lib, top_k=50, max_inflight=a.serve_inflight)
    build_s = time.perf_counter() - t0
    for L in pools:  # warm-up: first batches of every bucket, both extremes of q
        for n in (1, 512):
            srv.wait(srv.submit(pools[L][:n]))
    srv.wait_cluster(srv.submit_cluster(cjobs[0][:500], 3.0, 5))
    rate, T = a.serve_rate, a.serve_seconds
    st, lag, submit_s, n_req = _open_loop(srv, pools, shares, rate, T, rng, cjobs=cjobs)
    Ls = np.array([L for L, _ in shares])
    ps = np.array([p for _, p in shares])
    offered = float(rate * sum(ps[list(Ls).index(L)] * lib[L].shape[0] for L in Ls) * 256.5)
    open_loop = {"offered_req_per_s": rate, "seconds": T, "requests": n_req,
                 "cluster_jobs": len(cjobs), "offered_pairs_per_s": offered,
                 "p50_ms": st["p50_ms"], "p99_ms": st["p99_ms"], "max_ms": st["max_ms"], "mean_ms": st["mean_ms"],
                 "pairs_per_s": st["pairs_per_s"], "wall_s": st["seconds"], "batches": int(st["batches"]),
                 "mean_batch_rows": st["mean_batch_rows"], "plain_fallbacks": int(st["plain_fallbacks"]),
                 "cluster_p50_ms": st["cluster_p50_ms"], "cluster_p99_ms": st["cluster_p99_ms"],
                 "submit_lag_p99_ms": float(np.percentile(lag, 99)) if lag else None, "submit_s": submit_s,
                 "pairs_screened_per_pair": st["pairs_screened"] / max(st["pairs"], 1)}
    # the serving latency target is quoted for 64-structure queries: the same
    # Poisson load with every query exactly 64 structures
    st64, _, _, n64 = _open_loop(srv, pools, shares, rate, min(T, 2.0), rng, q_fixed=64)
    open_loop_q64 = {"offered_req_per_s": rate, "seconds": min(T, 2.0), "requests": n64, "q": 64,
                     "p50_ms": st64["p50_ms"], "p99_ms": st64["p99_ms"], "max_ms": st64["max_ms"],
                     "pairs_per_s": st64["pairs_per_s"]}
    cap = _closed_loop(srv, pools, shares, 2.0, rng)
    srv.close()
    # the plain FP64 server on the same library and GPU (closed loop)
    psrv = CrmsdServer(lib, top_k=50, max_inflight=2, precision="plain64")
    psrv.wait(psrv.submit(pools[64][:4]))
    pcap = _closed_loop(psrv, pools, shares, 2.0, rng, max_inflight=2)
    psrv.close()
    return {"library": {"structures": int(sum(x.shape[0] for x in lib.values())),
                        "atoms": int(sum(x.shape[0] * x.shape[1] for x in lib.values())),
                        "buckets": {str(L): int(lib[L].shape[0]) for L in lib}, "build_s": build_s},
            "top_k": 50, "max_inflight": a.serve_inflight, "open_loop": open_loop, "open_loop_q64": open_loop_q64,
            "capacity": {"pairs_per_s": cap["pairs_per_s"], "p50_ms": cap["p50_ms"], "p99_ms": cap["p99_ms"],
                         "queries": int(cap["queries_done"])},
            "plain64_capacity": {"pairs_per_s": pcap["pairs_per_s"], "p50_ms": pcap["p50_ms"],
                                 "p99_ms": pcap["p99_ms"], "queries": int(pcap["queries_done"])},
            "speedup_vs_plain64": cap["pairs_per_s"] / max(pcap["pairs_per_s"], 1.0)}


def run_reference(a, rank):
    if rank != 0:
        return
    w = workload(a)
    x = w.generate()
    samples = []
    for s in range(a.warmup + a.steps):
        cb = cpu_baseline(x, a.cpu_seconds / 2, seed=1000 + s)
        if s >= a.warmup:
            samples.append(cb)
    v = statistics.median([c["value"] for c in samples])
    cb = dict(samples[-1])
    cb["value"] = v
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": a.gpus, "steps": a.steps,
            "warmup": a.warmup, "ms_per_step": None, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": w.name, "n": w.n, "L": w.L, "pairs": w.pairs},
            "cpu_baseline": cb, "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(a, rank, world, local_rank):
    import torch
    from bioshell_gb300.crmsd import CrmsdOptions, Engine

    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist  # noqa: F811
        dist.init_process_group("nccl")
    w = workload(a)
    x, sig = w.generate(return_sigma=True)
    n, L = x.shape[0], x.shape[1]
    npairs = n * (n - 1) // 2
    eng = Engine(local_rank)
    stream = torch.cuda.ExternalStream(eng.stream_handle())
    xd = torch.from_numpy(x).cuda()
    outd = torch.empty(npairs, dtype=torch.float64, device="cuda")

    def barrier():
        torch.cuda.synchronize()
        if dist:
            dist.barrier()

    def step(xin, out, opts=None):
        eng.all_vs_all(xin, opts, out=out)
        return eng.metrics()

    # ---- device-resident timed region
    for _ in range(a.warmup):
        step(xd, outd)
    barrier()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    mets = []
    with Clocks(local_rank) as clk:
        ev0.record(stream)
        for _ in range(a.steps):
            mets.append(step(xd, outd))
        ev1.record(stream)
        ev1.synchronize()
    barrier()
    ms, value = whole_job_rate(ev0.elapsed_time(ev1), npairs, a.steps, world, dist)
    clocks = clk.summary()
    ms_main = statistics.mean(m["ms_main"] for m in mets)
    launches = int(sum(m["main_launches"] for m in mets))
    refined = mets[-1]["pairs_refined"]
    phases = {k: statistics.mean(m[k] for m in mets) for k in ("ms_prep", "ms_main", "ms_refine", "ms_total")}
    phases["quant_bound"] = mets[-1]["quant_bound"]
    phases["scale_exp"] = mets[-1]["scale_exp"]

    # ---- end to end through the C ABI with pinned host buffers
    xh = eng.host_empty(x.shape, np.float64)
    xh[...] = x
    oh = eng.host_empty((npairs,), np.float64)
    step(xh, oh)
    barrier()
    e_steps = max(1, min(a.steps, 3))
    ev0.record(stream)
    for _ in range(e_steps):
        step(xh, oh)
    ev1.record(stream)
    ev1.synchronize()
    ms_e2e, e2e_value = whole_job_rate(ev0.elapsed_time(ev1), npairs, e_steps, world, dist)
    # the machine's host link as a plain copy of the same triangle into the same
    # pinned buffer: an end-to-end step cannot take less than that copy
    ohv = torch.from_numpy(oh)
    torch.cuda.synchronize()
    l0, l1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    l0.record()
    ohv.copy_(outd, non_blocking=True)
    l1.record()
    l1.synchronize()
    link_gbs = npairs * 8 / (l0.elapsed_time(l1) * 1e-3) / 1e9
    e2e = {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(x.nbytes),
           "d2h_bytes_per_step": int(npairs * 8), "steps": e_steps, "ms_per_step": ms_e2e / e_steps,
           "host_link_d2h_gbs": link_gbs}
    np.testing.assert_array_equal(oh[:1000], outd[:1000].cpu().numpy())

    # ---- plain FP64 denominator on the same workload
    plain = None
    f64_flops = fp64_peak(local_rank) if rank == 0 else None
    if not a.skip_plain:
        step(xd, outd, CrmsdOptions(precision="plain64"))
        m = step(xd, outd, CrmsdOptions(precision="plain64"))
        plain = {"value": npairs / (m["ms_total"] * 1e-3), "unit": UNIT, "ms_per_step": m["ms_total"],
                 "kernel_ms": m["ms_main"]}
        if f64_flops:
            # algorithmic FP64 work: the covariance, 18 L flops per pair (the
            # per-pair QCP solve, ~200 flops, is not counted)
            ach = 18.0 * L * npairs / (m["ms_main"] * 1e-3)
            plain["roofline"] = {"kernel": "k_plain64_all", "bound": "fp64", "achieved_tflops": ach / 1e12,
                                 "peak_tflops": f64_flops / 1e12, "frac": ach / f64_flops,
                                 "peak_source": "measured in-tree (bs_diag_fp64_peak)"}
        step(xd, outd)  # leave the mixed result in outd

    # ---- accuracy against the FP64 oracle
    acc = None
    if not a.skip_accuracy and rank == 0:
        from oracle import oracle
        oracle.build()
        rng = np.random.default_rng(2024)
        sel = rng.choice(npairs, min(npairs, 1_000_000), replace=False)
        i, j = tri_pairs(n, sel)
        ref = oracle.crmsd_pairs(x, i, j, nthreads=host_threads())
        got = outd[torch.from_numpy(sel).cuda()].cpu().numpy()
        d = np.abs(got - ref)
        nd = np.flatnonzero(sig == w.near_dup_sigma)
        ia, ja = np.triu_indices(len(nd), 1)
        ni, nj = nd[ia], nd[ja]
        tsel = ni * n - ni * (ni + 1) // 2 + (nj - ni - 1)
        ref2 = oracle.crmsd_pairs(x, ni, nj, nthreads=host_threads())
        got2 = outd[torch.from_numpy(tsel).cuda()].cpu().numpy()
        d2 = np.abs(got2 - ref2)
        acc = {"random_pairs": int(len(sel)), "max_abs": float(d.max()), "p99_abs": float(np.percentile(d, 99)),
               "near_dup_pairs": int(len(tsel)), "near_dup_max_abs": float(d2.max()) if len(d2) else None,
               "near_dup_p99_abs": float(np.percentile(d2, 99)) if len(d2) else None,
               "tolerance": 1e-4, "pass": bool(d.max() <= 1e-4 and (len(d2) == 0 or d2.max() <= 1e-4))}

    neighbors = run_neighbors(eng, xd, outd, n, torch) if rank == 0 else None
    superpose = run_superpose(eng, xd, x, torch) if rank == 0 else None

    pk, pk_kind = peaks()
    achieved = 18.0 * L * npairs / (ms_main * 1e-3) / 1e12
    peak = pk["bf16_tflops_sustained"]
    traffic = profiled_traffic("mixed_tc")
    roof = {"kernel": "k_mixed_tc", "bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
            "frac": achieved / peak, "peak_source": f"{pk_kind} bf16 sustained",
            "issued_tflops": issued_flops(n, L) / (ms_main * 1e-3) / 1e12,
            "kernel_ms": ms_main, "traffic": traffic}
    # the preparation (centring, grid choice, digit rows): a streaming pass;
    # algorithmic bytes per structure: 24 L read (f64 xyz), 24 L written
    # (four bf16 digit rows of three coordinates), 40 B of per-structure data
    prep_bytes = float(n) * (48.0 * L + 40.0)
    prep_gbs = prep_bytes / (phases["ms_prep"] * 1e-3) / 1e9
    streaming = {"kernel": "k_mx_center/scale/norms/choose/digits (preparation)", "bound": "hbm",
                 "achieved": prep_gbs, "peak": pk["hbm_gbs"], "unit": "GB/s", "frac": prep_gbs / pk["hbm_gbs"],
                 "peak_source": f"{pk_kind} HBM copy", "bytes": prep_bytes, "ms": phases["ms_prep"],
                 "traffic": profiled_traffic("prep")}
    cb = cpu_baseline(x, a.cpu_seconds) if rank == 0 else None
    batched = serving = None
    if rank == 0 and not (a.skip_batched and a.skip_serving):
        del outd
        torch.cuda.empty_cache()
        eng.close()  # frees the 50k workspaces before the next sections
        eng = Engine(local_rank)
        stream = torch.cuda.ExternalStream(eng.stream_handle())
    formats = run_formats(eng, torch) if rank == 0 and not a.skip_batched else None
    hier = run_hierarchical(eng) if rank == 0 and not a.skip_batched else None
    if not a.skip_batched and rank == 0:
        batched = run_batched(a, eng, stream, torch)
    if not a.skip_serving and rank == 0:
        serving = run_serving(a)
    # The contract keys first, the large sections next, and the short headline
    # figures (accuracy, the plain FP64 denominator, serving latency) last, so
    # that the end of the line carries them.
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": a.steps, "warmup": a.warmup,
            "ms_per_step": ms / a.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "bf16", "data": "synthetic",
            "config": {"workload": w.name, "n": n, "L": L, "pairs": npairs, "precision": "mixed",
                       "output": "f64 packed triangle", "l2": "no flush: inputs (360 MB) and output (10 GB) exceed L2",
                       "replicas": world},
            "e2e": e2e, "gpu_launches": launches, "roofline": roof, "streaming_roofline": streaming,
            "cpu_baseline": cb, "clocks": clocks, "phases": phases,
            "neighbors": neighbors, "superpose": superpose, "formats": formats, "hierarchical": hier,
            "batched": batched, "serving": serving}
    if batched:
        line["batched_summary"] = {"value": batched["value"], "e2e": batched["e2e"]["value"],
                                   "speedup_vs_plain64": batched["speedup_vs_plain64"],
                                   "optics_identical": f"{batched['optics']['identical_labels']}/{batched['sets']}"}
    if serving:
        ol, q64 = serving["open_loop"], serving["open_loop_q64"]
        line["serving_summary"] = {"req_per_s": ol["offered_req_per_s"], "p50_ms": ol["p50_ms"], "p99_ms": ol["p99_ms"],
                                   "q64_p50_ms": q64["p50_ms"], "q64_p99_ms": q64["p99_ms"],
                                   "pairs_per_s": ol["pairs_per_s"],
                                   "speedup_vs_plain64": serving["speedup_vs_plain64"]}
    line["fp64_peak_tflops"] = f64_flops / 1e12 if f64_flops else None
    line["pairs_refined"] = int(refined)
    line["accuracy"] = acc
    line["plain64"] = plain
    line["speedup_vs_plain64"] = (value / world / plain["value"]) if plain else None
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def probe_serving(k):
    import time
    from bioshell_gb300 import CrmsdServer
    lib, bases = synth.serving_library()
    pools = synth.serving_queries(bases)
    srv = CrmsdServer(lib, top_k=50, max_inflight=1)
    srv.wait(srv.submit(pools[64][:256]))
    srv.reset_stats()
    t0 = time.perf_counter()
    for q in range(k):
        srv.wait(srv.submit(pools[64][(q * 64) % 768:(q * 64) % 768 + 256]))
    dt = time.perf_counter() - t0
    st = srv.stats()
    srv.close()
    print(json.dumps({"probe": "serving", "batches": k, "rows": 256, "library": int(lib[64].shape[0]),
                      "seconds": dt, "pairs_per_s": k * 256 * lib[64].shape[0] / dt, "p50_ms": st["p50_ms"]}))


def main():
    a = args_()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if a.impl == "reference":
        run_reference(a, rank)
        return
    if a.probe_serving > 0:
        probe_serving(a.probe_serving)
        return
    run_ours(a, rank, world, local_rank)


if __name__ == "__main__":
    main()
