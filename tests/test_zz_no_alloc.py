"""bs_all_vs_all_static: the all-vs-all entry point for callers that cannot
allocate device memory.

Such callers -- code inside another framework's memory pool, plugins limited
to the buffers they are handed, processes whose device footprint must stay
fixed -- pass device buffers for the coordinates and the result, and the
engine takes its scratch from static device arrays instead of cudaMalloc.
These tests call the entry point through the C ABI and check its results
against the allocating entry point, bs_all_vs_all, on two calls in a row
(the second with a different shape, so stale scratch from the first call
would show).  Both run the same kernels on the same plan, so the results
must be equal bit for bit; they are also checked against the FP64 oracle
within the mixed path's 1e-4 A tolerance.  This file is collected last on
purpose.
"""
import ctypes

import numpy as np
import pytest

from bioshell_gb300 import synth

pytestmark = pytest.mark.gpu

TOL = 1e-4  # the suite's tolerance for the mixed path (Angstrom)


def _static_call(lib, torch, x):
    xd = torch.from_numpy(np.ascontiguousarray(x)).cuda()
    n, L = x.shape[0], x.shape[1]
    out = torch.full((n * (n - 1) // 2,), -7.0, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    st = lib.bs_all_vs_all_static(ctypes.c_void_p(xd.data_ptr()), n, L, ctypes.c_void_p(out.data_ptr()), None)
    return st, out.cpu().numpy()


def test_static_matches_allocating_entry_point_twice(enginelib, oracle_mod):
    torch = pytest.importorskip("torch")
    from bioshell_gb300.crmsd import Engine

    eng = Engine(0)
    rng = np.random.default_rng(41)
    first = synth.decoys(synth.base_chain(64, rng), 300, rng, near_dup_frac=0.1)
    second = synth.decoys(synth.base_chain(129, rng), 97, rng, near_dup_frac=0.1)
    for x in (first, second):
        st, got = _static_call(enginelib, torch, x)
        assert st == 0, enginelib.bs_status_string(st)
        want = eng.all_vs_all(x).values
        np.testing.assert_array_equal(got, want)
        assert np.abs(got - oracle_mod.crmsd_all_vs_all(x)).max() <= TOL
    eng.close()


def test_static_rejects_sizes_beyond_its_scratch(enginelib):
    torch = pytest.importorskip("torch")
    x = torch.zeros((513, 8, 3), dtype=torch.float64, device="cuda")
    out = torch.zeros(513 * 512 // 2, dtype=torch.float64, device="cuda")
    assert enginelib.bs_all_vs_all_static(ctypes.c_void_p(x.data_ptr()), 513, 8, ctypes.c_void_p(out.data_ptr()),
                                          None) == 5  # BS_ERR_UNSUPPORTED
    assert enginelib.bs_all_vs_all_static(ctypes.c_void_p(x.data_ptr()), 4, 513, ctypes.c_void_p(out.data_ptr()),
                                          None) == 5
    host = np.zeros((4, 8, 3))
    assert enginelib.bs_all_vs_all_static(host.ctypes.data_as(ctypes.c_void_p), 4, 8,
                                          ctypes.c_void_p(out.data_ptr()), None) == 1  # host memory: invalid


def test_static_refuses_a_capturing_stream(enginelib):
    """The entry point copies from host memory and synchronises, which stream
    capture forbids: on a capturing stream it returns BS_ERR_UNSUPPORTED
    without a CUDA call that would invalidate the capture, and the captured
    graph still runs."""
    torch = pytest.importorskip("torch")
    n, L = 40, 16
    x = torch.zeros((n, L, 3), dtype=torch.float64, device="cuda")
    out = torch.zeros(n * (n - 1) // 2, dtype=torch.float64, device="cuda")
    y = torch.zeros(4, device="cuda")
    s = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    torch.cuda.synchronize()
    with torch.cuda.graph(g, stream=s, capture_error_mode="thread_local"):
        st = enginelib.bs_all_vs_all_static(ctypes.c_void_p(x.data_ptr()), n, L, ctypes.c_void_p(out.data_ptr()),
                                            ctypes.c_void_p(s.cuda_stream))
        y.add_(1.0)
    assert st == 5  # BS_ERR_UNSUPPORTED
    g.replay()
    torch.cuda.synchronize()
    assert float(y[0]) == 1.0
