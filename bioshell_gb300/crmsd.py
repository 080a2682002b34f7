"""Host-side API of the crmsd engine, mirroring the Rust interface the engine
is bound to in ``bioshell_pdb::calc``:

* ``crmsd(a, b)``                      -- one pair, ``&[T: HasCartesians]`` inputs
  (bioshell-core/src/has_cartesians.rs:6-8), like
  ``SubstructureAxis::from_3d_points`` (bioshell-pdb/src/calc/substructures.rs:17);
* ``crmsd_all_vs_all(models, opts)``   -- the distance matrix consumed by
  ``hierarchical_clustering`` (bioshell-clustering/src/hierarchical/
  hierarchical.rs:22) through ``HierarchicalClusteringMatrix::new``
  (clustering_matrix.rs:11-22), returned as a ``CrmsdMatrix``;
* ``crmsd_batched(sets, opts)``        -- one matrix per decoy set, all sets in one
  persistent tensor-core launch (the per-set clustering loop of a caller);
* ``CrmsdMatrix.get(i, j)`` / ``as_f32_closure()`` -- the ``Fn(usize, usize) -> f32``
  distance closure the clustering takes.

Everything computes on the GPU through the C ABI; there is no CPU path.
"""
from __future__ import annotations

import ctypes
import weakref
from dataclasses import dataclass
from typing import Optional

import numpy as np

from . import lib as _l


@dataclass
class CrmsdOptions:
    """Mirrors ``bs_opts``: precision ``"mixed"`` (tensor cores, default) or
    ``"plain64"``; layout ``"triangle"`` (packed upper triangle) or
    ``"square"``; element type ``"f64"`` or ``"f32"``; tolerance in Angstrom
    (None = engine default)."""

    precision: str = "mixed"
    layout: str = "triangle"
    out_type: str = "f64"
    tolerance: Optional[float] = None
    graph: bool = True  # replay a captured CUDA graph for repeated shapes
    autotune: bool = False  # time the tile shapes per set class (mixed path)
    flag_queue: int = 0  # capacity of the exact-recomputation queue (0 = default)
    rows: Optional[tuple] = None  # (row_begin, row_end): only the pairs of those rows (all_vs_all)

    def to_c(self) -> _l.bs_opts:
        o = _l.bs_opts()
        _l.load().bs_opts_init(ctypes.byref(o))
        o.precision = _l.PRECISION[self.precision]
        o.layout = _l.LAYOUT[self.layout]
        o.out_type = _l.OUT_TYPE[self.out_type]
        o.tolerance = float(self.tolerance or 0.0)
        o.flags = (0 if self.graph else _l.FLAG_NO_GRAPH) | (_l.FLAG_AUTOTUNE if self.autotune else 0)
        o.flag_queue = int(self.flag_queue)
        if self.rows is not None:
            o.row_begin, o.row_end = int(self.rows[0]), int(self.rows[1])
        return o


def partition_rows(n: int, parts: int):
    """Row bounds that split the pairs of an n-structure all-vs-all into
    `parts` ranges of nearly equal pair counts (bs_partition_rows): range p is
    CrmsdOptions(rows=(b[p], b[p + 1])), e.g. one per GPU."""
    b = np.zeros(parts + 1, dtype=np.int64)
    st = _l.load().bs_partition_rows(int(n), int(parts), b.ctypes.data)
    if st != _l.BS_OK:
        raise _l.CrmsdError(st, "bs_partition_rows")
    return b


def tri_index(n: int, i, j):
    """Index of pair (i, j), i < j, in the packed row-major upper triangle."""
    return i * n - i * (i + 1) // 2 + (j - i - 1)


class CrmsdMatrix:
    """All-vs-all crmsd values of n structures (packed triangle or square)."""

    def __init__(self, n: int, values, layout: str = "triangle"):
        self.n = n
        self.values = values
        self.layout = layout

    def get(self, i: int, j: int) -> float:
        if i == j:
            return 0.0
        if self.layout == "square":
            return float(self.values[i * self.n + j])
        if i > j:
            i, j = j, i
        return float(self.values[tri_index(self.n, i, j)])

    def as_f32_closure(self):
        """``Fn(usize, usize) -> f32`` for hierarchical_clustering."""
        v = self.values
        n = self.n
        if self.layout == "square":
            return lambda i, j: np.float32(v[i * n + j])
        return lambda i, j: np.float32(0.0) if i == j else np.float32(
            v[tri_index(n, min(i, j), max(i, j))])

    def to_square(self) -> np.ndarray:
        vals = np.asarray(self.values)
        if self.layout == "square":
            return vals.reshape(self.n, self.n)
        out = np.zeros((self.n, self.n), dtype=vals.dtype)
        iu = np.triu_indices(self.n, 1)
        out[iu] = vals
        out[(iu[1], iu[0])] = vals
        return out


def _ptr(x):
    """(address, keepalive) of a numpy array or a CUDA tensor."""
    if isinstance(x, np.ndarray):
        if not x.flags.c_contiguous:
            raise ValueError("arrays must be C-contiguous")
        return x.ctypes.data, x
    if hasattr(x, "data_ptr") and hasattr(x, "is_cuda"):
        if not x.is_contiguous():
            raise ValueError("tensors must be contiguous")
        return x.data_ptr(), x
    raise TypeError(f"unsupported buffer type {type(x)!r}")


class Engine:
    """A context on one GPU (``bs_ctx``): owns the stream and device workspaces."""

    def __init__(self, device: int = 0, hbm_budget: int = 0):
        self._lib = _l.load()
        h = ctypes.c_void_p()
        st = self._lib.bs_ctx_create(ctypes.byref(h), int(device), int(hbm_budget))
        if st != _l.BS_OK:
            raise _l.CrmsdError(st, "bs_ctx_create: " + self._lib.bs_status_string(st).decode())
        self._h = h
        self._fin = weakref.finalize(self, self._lib.bs_ctx_destroy, h)

    def close(self):
        self._fin()

    def _check(self, st: int):
        if st != _l.BS_OK:
            raise _l.CrmsdError(st, self._lib.bs_last_error(self._h).decode())

    def stream_handle(self) -> int:
        """The engine's cudaStream_t as an integer handle."""
        return int(self._lib.bs_ctx_stream(self._h) or 0)

    # -- metrics -------------------------------------------------------
    def metrics(self) -> dict:
        m = _l.bs_metrics()
        self._check(self._lib.bs_get_metrics(self._h, ctypes.byref(m)))
        return m.as_dict()

    # -- pinned host memory ----------------------------------------------
    def host_empty(self, shape, dtype=np.float64) -> np.ndarray:
        """numpy array backed by page-locked host memory."""
        dtype = np.dtype(dtype)
        nbytes = int(np.prod(shape)) * dtype.itemsize
        p = ctypes.c_void_p()
        self._check(self._lib.bs_host_alloc(max(nbytes, 1), ctypes.byref(p)))
        buf = (ctypes.c_char * max(nbytes, 1)).from_address(p.value)
        arr = np.frombuffer(buf, dtype=dtype, count=int(np.prod(shape))).reshape(shape)
        weakref.finalize(buf, self._lib.bs_host_free, ctypes.c_void_p(p.value))
        return arr

    # -- crmsd -------------------------------------------------------------
    def crmsd(self, a, b) -> float:
        a = np.ascontiguousarray(a, dtype=np.float64)
        b = np.ascontiguousarray(b, dtype=np.float64)
        if a.ndim != 2 or a.shape[1] != 3 or a.shape != b.shape:
            raise ValueError("crmsd: both inputs must be [L][3] with the same L")
        r = ctypes.c_double()
        self._check(self._lib.bs_crmsd(self._h, a.ctypes.data, b.ctypes.data, a.shape[0], ctypes.byref(r)))
        return r.value

    def all_vs_all(self, xyz, opts: Optional[CrmsdOptions] = None, out=None) -> CrmsdMatrix:
        opts = opts or CrmsdOptions()
        if isinstance(xyz, np.ndarray):
            xyz = np.ascontiguousarray(xyz, dtype=np.float64)
        if len(xyz.shape) != 3 or xyz.shape[2] != 3:
            raise ValueError("coordinates must be [n][L][3]")
        n, L = int(xyz.shape[0]), int(xyz.shape[1])
        count = n * (n - 1) // 2 if opts.layout == "triangle" else n * n
        dt = np.float64 if opts.out_type == "f64" else np.float32
        if out is None:
            out = np.empty(count, dtype=dt)
        xp, _k1 = _ptr(xyz)
        op, _k2 = _ptr(out)
        o = opts.to_c()
        self._check(self._lib.bs_all_vs_all(self._h, xp, n, L, ctypes.byref(o), op))
        return CrmsdMatrix(n, out, opts.layout)

    def neighbors(self, xyz, eps: float, opts: Optional[CrmsdOptions] = None):
        """eps-neighbour lists without the dense matrix: CSR (row_ptr int64
        [n+1], col int32, dist f32); row i holds every j != i with crmsd <= eps,
        ordered by (crmsd, j).  Feed them to ``clustering.optics_neighbors``."""
        opts = opts or CrmsdOptions()
        if isinstance(xyz, np.ndarray):
            xyz = np.ascontiguousarray(xyz, dtype=np.float64)
        if len(xyz.shape) != 3 or xyz.shape[2] != 3:
            raise ValueError("coordinates must be [n][L][3]")
        n, L = int(xyz.shape[0]), int(xyz.shape[1])
        xp, _k1 = _ptr(xyz)
        o = opts.to_c()
        nnz = ctypes.c_int64()
        self._check(self._lib.bs_neighbors(self._h, xp, n, L, float(eps), ctypes.byref(o), ctypes.byref(nnz)))
        row_ptr = np.zeros(n + 1, dtype=np.int64)
        col = np.zeros(nnz.value, dtype=np.int32)
        dist = np.zeros(nnz.value, dtype=np.float32)
        self._check(self._lib.bs_neighbors_get(self._h, row_ptr.ctypes.data, col.ctypes.data, dist.ctypes.data))
        return row_ptr, col, dist

    def batched(self, sets, opts: Optional[CrmsdOptions] = None, outs=None):
        """All-vs-all of every set in ``sets`` (each [n][L][3], numpy or CUDA
        tensor; n and L may differ) in one call; returns one CrmsdMatrix per set."""
        opts = opts or CrmsdOptions()
        dt = np.float64 if opts.out_type == "f64" else np.float32
        descs = (_l.bs_set_desc * max(len(sets), 1))()
        keep = []
        mats = []
        for k, x in enumerate(sets):
            if isinstance(x, np.ndarray):
                x = np.ascontiguousarray(x, dtype=np.float64)
            if len(x.shape) != 3 or x.shape[2] != 3:
                raise ValueError("each set must be [n][L][3]")
            n, L = int(x.shape[0]), int(x.shape[1])
            count = n * (n - 1) // 2 if opts.layout == "triangle" else n * n
            out = outs[k] if outs is not None else np.empty(count, dtype=dt)
            xp, k1 = _ptr(x)
            op, k2 = _ptr(out)
            keep += [k1, k2]
            descs[k].xyz = xp
            descs[k].n = n
            descs[k].L = L
            descs[k].out = op
            mats.append(CrmsdMatrix(n, out, opts.layout))
        o = opts.to_c()
        self._check(self._lib.bs_batched(self._h, descs, len(sets), ctypes.byref(o)))
        return mats

    def tile_shape(self, L: int, n: int):
        """The autotuner's choice for sets of L atoms and n structures:
        "narrow" (40 x 10 tiles), "wide" (40 x 20), or None if not timed."""
        v = ctypes.c_int32()
        self._check(self._lib.bs_tune_get(self._h, int(L), int(n), ctypes.byref(v)))
        return None if v.value < 0 else ("narrow" if v.value else "wide")

    def set_tile_shape(self, L: int, n: int, shape: str):
        self._check(self._lib.bs_tune_set(self._h, int(L), int(n), 1 if shape == "narrow" else 0))

    def tuning(self) -> dict:
        """The autotuner's cache: {"num_sms": N, "classes": [[L, n, "wide"|"narrow"], ...]}
        with (L, n) a representative chain length and set size of each class."""
        cnt, sms = ctypes.c_int32(), ctypes.c_int32()
        self._check(self._lib.bs_tune_list(self._h, None, None, None, 0, ctypes.byref(cnt), ctypes.byref(sms)))
        k = cnt.value
        Ls, ns, nw = np.zeros(k, np.int32), np.zeros(k, np.int64), np.zeros(k, np.int32)
        self._check(self._lib.bs_tune_list(self._h, Ls.ctypes.data, ns.ctypes.data, nw.ctypes.data, k,
                                           ctypes.byref(cnt), ctypes.byref(sms)))
        return {"num_sms": int(sms.value),
                "classes": [[int(a), int(b), "narrow" if c else "wide"] for a, b, c in zip(Ls, ns, nw)]}

    def save_tuning(self, path: str):
        """Writes the autotuner's cache as JSON, keyed by the GPU's SM count."""
        import json
        with open(path, "w") as fh:
            json.dump(self.tuning(), fh)

    def load_tuning(self, path: str) -> bool:
        """Restores a cache saved on a GPU with the same SM count (False, and
        nothing loaded, for another SM count)."""
        import json
        with open(path) as fh:
            t = json.load(fh)
        if int(t.get("num_sms", -1)) != self.tuning()["num_sms"]:
            return False
        for L, n, shape in t["classes"]:
            self.set_tile_shape(L, n, shape)
        return True

    def pairs(self, xyz, ii, jj, opts: Optional[CrmsdOptions] = None, out=None):
        opts = opts or CrmsdOptions()
        if isinstance(xyz, np.ndarray):
            xyz = np.ascontiguousarray(xyz, dtype=np.float64)
        n, L = int(xyz.shape[0]), int(xyz.shape[1])
        if isinstance(ii, np.ndarray) or not hasattr(ii, "data_ptr"):
            ii = np.ascontiguousarray(ii, dtype=np.int64)
            jj = np.ascontiguousarray(jj, dtype=np.int64)
        npairs = int(ii.shape[0])
        if out is None:
            out = np.empty(npairs, dtype=np.float64)
        xp, _k1 = _ptr(xyz)
        ip, _k2 = _ptr(ii)
        jp, _k3 = _ptr(jj)
        op, _k4 = _ptr(out)
        o = opts.to_c()
        self._check(self._lib.bs_pairs(self._h, xp, n, L, ip, jp, npairs, ctypes.byref(o), op))
        return out

    # -- superposition -------------------------------------------------------
    def superpose(self, a, b):
        """The superposition of b onto a: (Rototranslation with R b + t ~ a,
        RMSD of that superposition)."""
        from .superpose import Rototranslation

        a = np.ascontiguousarray(a, dtype=np.float64)
        b = np.ascontiguousarray(b, dtype=np.float64)
        if a.ndim != 2 or a.shape[1] != 3 or a.shape != b.shape:
            raise ValueError("superpose: both inputs must be [L][3] with the same L")
        rot = np.empty(9)
        t = np.empty(3)
        r = np.empty(1)
        self._check(self._lib.bs_superpose(self._h, a.ctypes.data, b.ctypes.data, a.shape[0], rot.ctypes.data,
                                           t.ctypes.data, r.ctypes.data))
        return Rototranslation(rot.reshape(3, 3), t), float(r[0])

    def superpose_pairs(self, xyz, ii, jj, out=None):
        """For each pair t: rot[t] (3x3), trans[t] (3) with rot x_jj[t] + trans ~
        x_ii[t], and the RMSD of that superposition.  xyz ([n][L][3]) and the
        pair lists may be numpy arrays or CUDA tensors; ``out`` = (rot, trans,
        rmsd) buffers (numpy or CUDA), allocated on the host when omitted."""
        if isinstance(xyz, np.ndarray) or not hasattr(xyz, "data_ptr"):
            xyz = np.ascontiguousarray(xyz, dtype=np.float64)
        if len(xyz.shape) != 3 or xyz.shape[2] != 3:
            raise ValueError("coordinates must be [n][L][3]")
        n, L = int(xyz.shape[0]), int(xyz.shape[1])
        if isinstance(ii, np.ndarray) or not hasattr(ii, "data_ptr"):
            ii = np.ascontiguousarray(ii, dtype=np.int64)
            jj = np.ascontiguousarray(jj, dtype=np.int64)
        if tuple(ii.shape) != tuple(jj.shape) or len(ii.shape) != 1:
            raise ValueError("pair lists must be 1-D and of equal length")
        npairs = int(ii.shape[0])
        if out is None:
            out = (np.empty((npairs, 3, 3)), np.empty((npairs, 3)), np.empty(npairs))
        rot, trans, rmsd = out
        if npairs:
            xp, _k1 = _ptr(xyz)
            ip, _k2 = _ptr(ii)
            jp, _k3 = _ptr(jj)
            rp, _k4 = _ptr(rot)
            tp, _k5 = _ptr(trans)
            mp, _k6 = _ptr(rmsd)
            self._check(self._lib.bs_superpose_pairs(self._h, xp, n, L, ip, jp, npairs, rp, tp, mp))
        return rot, trans, rmsd

    # -- diagnostics ---------------------------------------------------------
    def debug_tile_levels(self, xyz) -> np.ndarray:
        xyz = np.ascontiguousarray(xyz, dtype=np.float64)
        out = np.zeros((4, 128, 128), dtype=np.float32)
        self._check(self._lib.bs_debug_tile_levels(self._h, xyz.ctypes.data, xyz.shape[0], xyz.shape[1],
                                                   out.ctypes.data_as(ctypes.POINTER(ctypes.c_float))))
        return out

    def debug_pair_levels(self, xyz, ii, jj):
        xyz = np.ascontiguousarray(xyz, dtype=np.float64)
        ii = np.ascontiguousarray(ii, dtype=np.int64)
        jj = np.ascontiguousarray(jj, dtype=np.int64)
        lv = np.zeros((ii.shape[0], 4, 9), dtype=np.float32)
        r = np.zeros(ii.shape[0])
        self._check(self._lib.bs_debug_pair_levels(self._h, xyz.ctypes.data, xyz.shape[0], xyz.shape[1],
                                                   ii.ctypes.data, jj.ctypes.data, ii.shape[0],
                                                   lv.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                                   r.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
        return lv, r


_default: Optional[Engine] = None


def default_engine() -> Engine:
    global _default
    if _default is None:
        _default = Engine(0)
    return _default


def crmsd(a, b) -> float:
    """crmsd of two index-matched [L][3] coordinate sets (on the GPU)."""
    return default_engine().crmsd(a, b)


def superpose(a, b):
    """(Rototranslation moving b onto a, its RMSD), on the GPU."""
    return default_engine().superpose(a, b)


def crmsd_all_vs_all(models, opts: Optional[CrmsdOptions] = None) -> CrmsdMatrix:
    """All-vs-all crmsd of ``models`` ([n][L][3], or a list of [L][3])."""
    if isinstance(models, (list, tuple)):
        models = np.stack([np.asarray(m, dtype=np.float64) for m in models])
    return default_engine().all_vs_all(models, opts)


def crmsd_batched(sets, opts: Optional[CrmsdOptions] = None):
    """All-vs-all crmsd of every decoy set in ``sets``: a list of CrmsdMatrix."""
    return default_engine().batched(sets, opts)
