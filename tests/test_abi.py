"""The C ABI boundary: the library loads, exports every entry point the header
declares, its structs match the ctypes mirror, and on a machine without a
GPU it refuses compute instead of falling back to the CPU."""
import ctypes
import os
import re
import subprocess
import tempfile

import pytest

from bioshell_gb300 import lib as L

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "bioshell_crmsd.h")


def declared_functions():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"BS_API\s+[\w\s\*]*?\b(bs_\w+)\s*\(", text)))


def test_header_declares_entry_points():
    names = declared_functions()
    for must in ("bs_ctx_create", "bs_ctx_destroy", "bs_all_vs_all", "bs_pairs", "bs_crmsd", "bs_last_error"):
        assert must in names


def test_library_exports_every_declared_symbol(enginelib):
    for name in declared_functions():
        assert hasattr(enginelib, name), f"{name} declared in the header but not exported"


def test_ctypes_signatures_cover_header():
    bound = {s[0] for s in L.SIGNATURES}
    assert set(declared_functions()) == bound


def test_abi_version_and_status_strings(enginelib):
    assert enginelib.bs_abi_version() == 3
    assert enginelib.bs_status_string(0) == b"ok"
    assert enginelib.bs_status_string(8).startswith(b"no usable")
    assert enginelib.bs_status_string(1234) == b"unknown status"


def test_opts_init(enginelib):
    o = L.bs_opts()
    enginelib.bs_opts_init(ctypes.byref(o))
    assert o.version == 1 and o.precision == 1 and o.layout == 0 and o.out_type == 0


def test_struct_layout_matches_c():
    src = r"""
#include <stdio.h>
#include <stddef.h>
#include "bioshell_crmsd.h"
int main(void) {
  printf("%zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu\n", sizeof(bs_opts), offsetof(bs_opts, tolerance),
         offsetof(bs_opts, flags), sizeof(bs_metrics), offsetof(bs_metrics, scale_exp),
         offsetof(bs_metrics, graph), offsetof(bs_metrics, quant_bound), offsetof(bs_metrics, bytes_d2h),
         sizeof(bs_set_desc), offsetof(bs_set_desc, L), offsetof(bs_set_desc, out));
  return 0;
}
"""
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "t.c")
        exe = os.path.join(d, "t")
        open(c, "w").write(src)
        subprocess.run(["gcc", "-std=c99", "-I", os.path.dirname(HEADER), c, "-o", exe], check=True)
        got = [int(v) for v in subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()]
    want = [ctypes.sizeof(L.bs_opts), L.bs_opts.tolerance.offset, L.bs_opts.flags.offset,
            ctypes.sizeof(L.bs_metrics), L.bs_metrics.scale_exp.offset, L.bs_metrics.graph.offset,
            L.bs_metrics.quant_bound.offset, L.bs_metrics.bytes_d2h.offset, ctypes.sizeof(L.bs_set_desc),
            L.bs_set_desc.L.offset, L.bs_set_desc.out.offset]
    assert got == want


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.mark.skipif(_has_gpu(), reason="checks the no-GPU refusal")
def test_no_gpu_means_no_compute(enginelib):
    h = ctypes.c_void_p()
    assert enginelib.bs_ctx_create(ctypes.byref(h), 0, 0) == 8  # BS_ERR_NO_DEVICE
    from bioshell_gb300.crmsd import Engine
    with pytest.raises(L.CrmsdError):
        Engine(0)


def test_null_context_is_rejected(enginelib):
    assert enginelib.bs_all_vs_all(None, None, 0, 1, None, None) == 1
    assert enginelib.bs_ctx_create(None, 0, 0) == 1
    assert enginelib.bs_last_error(None) == b"null context"


def test_partition_rows_balances_pairs(enginelib):
    """bs_partition_rows: bounds from 0 to n, inner bounds on 40-structure
    blocks, and ranges whose pair counts differ by at most one block row."""
    from bioshell_gb300.crmsd import partition_rows
    for n, parts in ((50000, 8), (20000, 3), (1000, 4), (39, 2), (0, 1)):
        b = partition_rows(n, parts)
        assert b[0] == 0 and b[-1] == n and all(b[k] <= b[k + 1] for k in range(parts))
        assert all(v % 40 == 0 or v == n for v in b[1:-1])
        off = [int(r) * n - int(r) * (int(r) + 1) // 2 for r in b]
        counts = [off[k + 1] - off[k] for k in range(parts)]
        assert sum(counts) == n * (n - 1) // 2
        if n >= 1000:  # one block row holds at most 40 (n - 1) pairs
            assert max(counts) - min(counts) <= 2 * 40 * n
    assert enginelib.bs_partition_rows(10, 0, None) == 1
