"""CPU oracles for the crmsd path -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline legs of
``bench.py`` import this module.  The product library never does.

Two independent FP64 methods are exposed:

* ``crmsd_*`` -- the C restatement of the QCP method (``crmsd_oracle.c``);
  this is the oracle every GPU result is compared against.
* ``kabsch_*`` -- an SVD-Kabsch in numpy (determinant sign fix for proper
  rotations), used only to pin the QCP oracle itself.

The reference (BioShell 4.0.0-dev) has no crmsd routine to pin against
(bioshell-pdb/src/calc/mod.rs:1-10 exports none; bioshell-pdb/Cargo.toml:27
only mentions it).  Parity of the crmsd values with the reference is therefore
unpinned; the tests pin the oracle with analytic known answers and the SVD
cross-check.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libcrmsd_oracle.so")
_lib = None
_lock = threading.Lock()


def build() -> str:
    """Compile the C oracle with its Makefile (portable flags)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def _load():
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        src = os.path.join(_HERE, "crmsd_oracle.c")
        if not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(src):
            build()
        lib = ctypes.CDLL(_LIB_PATH)
        dp = ctypes.POINTER(ctypes.c_double)
        i64p = ctypes.POINTER(ctypes.c_int64)
        lib.bs_oracle_crmsd.restype = ctypes.c_double
        lib.bs_oracle_crmsd.argtypes = [dp, dp, ctypes.c_int]
        lib.bs_oracle_pair_terms.restype = None
        lib.bs_oracle_pair_terms.argtypes = [dp, dp, ctypes.c_int, dp]
        lib.bs_oracle_all_vs_all.restype = ctypes.c_int
        lib.bs_oracle_all_vs_all.argtypes = [dp, ctypes.c_int64, ctypes.c_int, dp, ctypes.c_int]
        lib.bs_oracle_pairs.restype = ctypes.c_int
        lib.bs_oracle_pairs.argtypes = [dp, ctypes.c_int64, ctypes.c_int, i64p, i64p, ctypes.c_int64, dp,
                                        ctypes.c_int]
        _lib = lib
        return lib


def _dptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _default_threads() -> int:
    return max(1, len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count() or 1)


def crmsd(a: np.ndarray, b: np.ndarray) -> float:
    """FP64 QCP crmsd of two index-matched [L][3] coordinate sets."""
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    if a.shape != b.shape or a.ndim != 2 or a.shape[1] != 3:
        raise ValueError("crmsd: both inputs must be [L][3] with the same L")
    return float(_load().bs_oracle_crmsd(_dptr(a), _dptr(b), a.shape[0]))


def pair_terms(a: np.ndarray, b: np.ndarray):
    """(lambda_max, G_a, G_b, rmsd) of one pair, from the FP64 QCP oracle."""
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    out = np.zeros(4)
    _load().bs_oracle_pair_terms(_dptr(a), _dptr(b), a.shape[0], _dptr(out))
    return tuple(out)


def crmsd_all_vs_all(xyz: np.ndarray, nthreads: int | None = None) -> np.ndarray:
    """Packed upper triangle (row-major, no diagonal) of FP64 crmsd values."""
    xyz = np.ascontiguousarray(xyz, dtype=np.float64)
    n, L, _ = xyz.shape
    out = np.empty(n * (n - 1) // 2, dtype=np.float64)
    rc = _load().bs_oracle_all_vs_all(_dptr(xyz), n, L, _dptr(out), nthreads or _default_threads())
    if rc != 0:
        raise RuntimeError(f"oracle all_vs_all failed: {rc}")
    return out


def crmsd_pairs(xyz: np.ndarray, ii: np.ndarray, jj: np.ndarray, nthreads: int | None = None) -> np.ndarray:
    """FP64 crmsd of an explicit list of pairs (ii[t], jj[t])."""
    xyz = np.ascontiguousarray(xyz, dtype=np.float64)
    ii = np.ascontiguousarray(ii, dtype=np.int64)
    jj = np.ascontiguousarray(jj, dtype=np.int64)
    n, L, _ = xyz.shape
    out = np.empty(ii.shape[0], dtype=np.float64)
    i64p = ctypes.POINTER(ctypes.c_int64)
    rc = _load().bs_oracle_pairs(_dptr(xyz), n, L, ii.ctypes.data_as(i64p), jj.ctypes.data_as(i64p),
                                 ii.shape[0], _dptr(out), nthreads or _default_threads())
    if rc != 0:
        raise RuntimeError(f"oracle pairs failed: {rc}")
    return out


# --------------------------------------------------------------------------
# Independent second oracle: SVD-Kabsch (numpy), used only to pin the QCP one
# --------------------------------------------------------------------------
def kabsch_pairs(xyz: np.ndarray, ii: np.ndarray, jj: np.ndarray) -> np.ndarray:
    """FP64 RMSD after optimal proper superposition, via batched 3x3 SVD."""
    xyz = np.asarray(xyz, dtype=np.float64)
    cen = xyz - xyz.mean(axis=1, keepdims=True)
    g = np.einsum("nkd,nkd->n", cen, cen)
    a = cen[ii]
    b = cen[jj]
    s = np.einsum("pkx,pky->pxy", a, b)
    sv = np.linalg.svd(s, compute_uv=False)
    sign = np.sign(np.linalg.det(s))
    sign[sign == 0] = 1.0
    trace = sv[:, 0] + sv[:, 1] + sign * sv[:, 2]
    e = (g[ii] + g[jj] - 2.0 * trace) / xyz.shape[1]
    return np.sqrt(np.maximum(e, 0.0))


def kabsch_superpose(a: np.ndarray, b: np.ndarray):
    """Optimal proper superposition of b onto a by SVD-Kabsch, as the
    (rotation, translation) pair a Rototranslation carries
    (bioshell-pdb/src/calc/transformation.rs:22-37; applied as R v + t by
    apply_mut, :171-174): R (3x3) and t with R b_k + t ~ a_k.  Returns
    (R, t, rmsd of that superposition)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    ca, cb = a.mean(axis=0), b.mean(axis=0)
    h = (b - cb).T @ (a - ca)  # sum_k (b_k - cb)(a_k - ca)^T
    u, _, vt = np.linalg.svd(h)
    d = 1.0 if np.linalg.det(vt.T @ u.T) >= 0 else -1.0
    r = vt.T @ np.diag([1.0, 1.0, d]) @ u.T
    t = ca - r @ cb
    res = b @ r.T + t - a
    return r, t, float(np.sqrt((res * res).sum() / a.shape[0]))


def tri_index(n: int, i, j):
    """Index of pair (i, j), i < j, in the packed row-major upper triangle."""
    i = np.asarray(i, dtype=np.int64)
    j = np.asarray(j, dtype=np.int64)
    return i * n - i * (i + 1) // 2 + (j - i - 1)
