"""Row bands of the banded read-back (host logic, no GPU).

A result of many pairs copied into host memory is read back in row bands:
each band is copied while later bands still compute.  The bands must cover
the packed triangle exactly once, in order, end on whole super-rows (32
blocks of 40 structures, the unit of the tile order), hold about 1/16 of
the pairs each, and taper at the end so the last copy -- which no
computation hides -- is short.
"""
import ctypes

import numpy as np
import pytest

SUPER_ROW = 32 * 40  # structures per super-row of the tile order


def _bands(lib, n, bands=16, cap=64):
    ends = np.zeros(cap, dtype=np.int64)
    count = ctypes.c_int32()
    st = lib.bs_selftest_bands(n, bands, ends.ctypes.data, cap, ctypes.byref(count))
    assert st == 0
    return ends[:count.value]


def _row_start(n, r):  # packed index of pair (r, r + 1)
    return r * n - r * (r + 1) // 2


@pytest.mark.parametrize("n", [20_000, 50_000, 100_000])
def test_bands_cover_the_triangle_and_taper(enginelib, n):
    ends = _bands(enginelib, n)
    total = n * (n - 1) // 2
    assert ends[-1] == total
    assert np.all(np.diff(ends) > 0)
    starts = {_row_start(n, r) for r in range(0, n, SUPER_ROW)}
    assert all(int(e) in starts for e in ends[:-1])  # whole super-rows
    sizes = np.diff(np.concatenate([[0], ends]))
    want = total // 16
    # a band is cut at the first super-row boundary past its target: equal
    # targets while more than two bands' worth is left, so those bands hold
    # at least 1/16 of the pairs and at most one super-row more
    for k, size in enumerate(sizes[:-1]):
        if total - (ends[k] - size) > 2 * want:
            assert want <= size <= want + SUPER_ROW * n
    # the tail halves down: the last band is a small fraction of a full one
    assert sizes[-1] <= want // 8
    assert len(ends) <= 16 + 8


def test_bands_of_small_sets(enginelib):
    for n in (2, 41, 1281, 5000):
        ends = _bands(enginelib, n)
        assert ends[-1] == n * (n - 1) // 2
        assert np.all(np.diff(ends) > 0)


def test_bands_reject_bad_arguments(enginelib):
    ends = np.zeros(4, dtype=np.int64)
    count = ctypes.c_int32()
    assert enginelib.bs_selftest_bands(1, 16, ends.ctypes.data, 4, ctypes.byref(count)) == 1
    assert enginelib.bs_selftest_bands(100, 0, ends.ctypes.data, 4, ctypes.byref(count)) == 1
    # more bands than the caller's array holds
    assert enginelib.bs_selftest_bands(50_000, 16, ends.ctypes.data, 4, ctypes.byref(count)) == 1
