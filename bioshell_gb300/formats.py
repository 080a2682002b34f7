"""The data formats either side of the crmsd path, through the C ABI:

* ``read_models(path, ca_only)``  -- every model of a PDB or mmCIF file as a
  ``[n_models][L][3]`` f64 array (bioshell-pdb's model_coordinates, read in
  one pass; ``bs_models_read``);
* ``write_tsv(path, matrix, labels)`` / ``read_tsv(path)`` -- the distance
  matrix TSV the clust tool reads (``bs_tsv_write`` / ``bs_tsv_read``).
"""
import ctypes
from typing import Optional, Sequence

import numpy as np

from . import lib as _l
from .crmsd import CrmsdMatrix


class FormatError(RuntimeError):
    def __init__(self, status: int, what: str):
        super().__init__(f"{what}: status {status}: {_l.load().bs_io_last_error().decode()}")
        self.status = status


def read_models(path: str, ca_only: bool = False, fmt: str = "auto") -> np.ndarray:
    lib = _l.load()
    h = ctypes.c_void_p()
    n, L = ctypes.c_int64(), ctypes.c_int32()
    code = {"auto": 0, "pdb": 1, "cif": 2}[fmt]
    st = lib.bs_models_read(path.encode(), code, 1 if ca_only else 0, ctypes.byref(h), ctypes.byref(n), ctypes.byref(L))
    if st:
        raise FormatError(st, "bs_models_read")
    try:
        out = np.empty((n.value, L.value, 3), dtype=np.float64)
        st = lib.bs_models_copy(h, out.ctypes.data)
        if st:
            raise FormatError(st, "bs_models_copy")
    finally:
        lib.bs_models_free(h)
    return out


def write_tsv(path: str, matrix, labels: Optional[Sequence[str]] = None, decimals: int = 6, n: Optional[int] = None):
    """Writes a packed triangle (CrmsdMatrix, numpy array or CUDA tensor)."""
    lib = _l.load()
    if isinstance(matrix, CrmsdMatrix):
        if matrix.layout != "triangle":
            raise ValueError("write_tsv takes the packed triangle layout")
        n, vals = matrix.n, matrix.values
    else:
        vals = matrix
        if n is None:
            m = int(vals.shape[0])
            n = int(round((1 + (1 + 8 * m) ** 0.5) / 2))
    if isinstance(vals, np.ndarray):
        vals = np.ascontiguousarray(vals)
        ptr, ot = vals.ctypes.data, (0 if vals.dtype == np.float64 else 1)
    else:  # CUDA tensor
        ptr, ot = vals.data_ptr(), (0 if str(vals.dtype) == "torch.float64" else 1)
    arr = None
    if labels is not None:
        enc = [str(s).encode() for s in labels]
        arr = (ctypes.c_char_p * len(enc))(*enc)
    st = lib.bs_tsv_write(path.encode(), ptr, n, ot, arr, decimals)
    if st:
        raise FormatError(st, "bs_tsv_write")


def read_tsv(path: str, default: float = 100.0, symmetric: bool = True):
    """(labels, CrmsdMatrix of f32 values in the packed triangle)."""
    lib = _l.load()
    h = ctypes.c_void_p()
    n = ctypes.c_int64()
    st = lib.bs_tsv_read(path.encode(), float(default), 1 if symmetric else 0, ctypes.byref(h), ctypes.byref(n))
    if st:
        raise FormatError(st, "bs_tsv_read")
    try:
        m = n.value
        tri = np.empty(m * (m - 1) // 2, dtype=np.float32)
        st = lib.bs_tsv_matrix(h, tri.ctypes.data_as(ctypes.POINTER(ctypes.c_float)))
        if st:
            raise FormatError(st, "bs_tsv_matrix")
        labels = [lib.bs_tsv_label(h, i).decode() for i in range(m)]
    finally:
        lib.bs_tsv_free(h)
    return labels, CrmsdMatrix(m, tri, "triangle")
