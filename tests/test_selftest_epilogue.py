"""CPU checks of the mixed path's fixed-point algebra, through the library's
host-side self-test hooks (the same crmsd_math.cuh code the kernels run).

Level sums are formed here exactly (numpy int64), exactly as the tensor-core
accumulators hold them; the fast epilogue and the exact recomputation must
then reproduce the FP64 oracle within the engine's error budget: quantisation
(each structure's RMS residual, summed over the pair) plus the fast path's
certified tolerance.
"""
import ctypes

import numpy as np
import pytest

from bioshell_gb300 import synth

TOL_TOTAL = 1e-4  # certified |dRMSD| per pair (Angstrom): quantisation + fast-path arithmetic


def _grid_exp(xs):
    m = max(np.abs(x - x.mean(0)).max() for x in xs)
    e = int(np.ceil(np.log2(m / (2 ** 22 - 1))))
    while np.ldexp(2 ** 22 - 1, e) < m:
        e += 1
    while np.ldexp(2 ** 22 - 1, e - 1) >= m:
        e -= 1
    return e


def join(d):
    """Quantised coordinates from stored digits: n = 2^14 e0 + 2^5 e1 + e2 / 16."""
    return d[0] * 16384 + d[1] * 32 + d[2] // 16


class Hooks:
    def __init__(self, lib):
        self.lib = lib

    def digits(self, x, e):
        L = x.shape[0]
        d = np.zeros((3, 3, L), dtype=np.int32)
        g, q = ctypes.c_int64(), ctypes.c_double()
        x = np.ascontiguousarray(x, dtype=np.float64)
        st = self.lib.bs_selftest_digits(x.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), L, e,
                                         d.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), ctypes.byref(g),
                                         ctypes.byref(q))
        assert st == 0
        return d.astype(np.int64), g.value, q.value

    @staticmethod
    def levels(da, db):
        """Level sums as the tensor cores hold them: 0-2 exact, 3 = S3 + S4/512."""
        s = np.zeros((4, 3, 3), dtype=np.float64)
        for x in range(3):
            for y in range(3):
                a, b = da[:, x, :], db[:, y, :]
                s[0, x, y] = (a[0] * b[0]).sum()
                s[1, x, y] = (a[0] * b[1] + a[1] * b[0]).sum()
                s[2, x, y] = (a[0] * b[2] + a[1] * b[1] + a[2] * b[0]).sum()
                s[3, x, y] = (a[1] * b[2] + a[2] * b[1]).sum() + (a[2] * b[2]).sum() / 512.0
        return s

    def fast(self, s, ga, gb, qa, qb, e, L, tol=TOL_TOTAL):
        lv = np.ascontiguousarray(s.reshape(4, 9), dtype=np.float32)
        # one rounding of level 3 to float: <= half an ulp of its magnitude
        top = np.abs(s[3]).max()
        d34 = 0.0 if top < 2 ** 23 else 12 * np.sqrt(3) * 2.0 ** (np.floor(np.log2(top)) - 24)
        r, f = ctypes.c_double(), ctypes.c_int32()
        st = self.lib.bs_selftest_epilogue(lv.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), ga, gb, qa, qb, d34,
                                           e, L, tol, ctypes.byref(r), ctypes.byref(f))
        assert st == 0
        return r.value, f.value

    def exact(self, da, db, e):
        na = np.ascontiguousarray(join(da).astype(np.int32))
        nb = np.ascontiguousarray(join(db).astype(np.int32))
        r = ctypes.c_double()
        p = ctypes.POINTER(ctypes.c_int32)
        st = self.lib.bs_selftest_exact(na.ctypes.data_as(p), nb.ctypes.data_as(p), na.shape[1], e, ctypes.byref(r))
        assert st == 0
        return r.value


@pytest.fixture(scope="module")
def hooks(enginelib):
    return Hooks(enginelib)


def test_digits_reconstruct(hooks):
    rng = np.random.default_rng(1)
    x = rng.normal(size=(50, 3)) * 20
    e = _grid_exp([x])
    d, g, q = hooks.digits(x, e)
    assert np.abs(d).max() <= 256 and np.all(d[2] % 16 == 0) and np.abs(d[2]).max() <= 256
    n = join(d)
    y = x - x.mean(0)
    assert np.abs(n.T * 2.0 ** e - y).max() <= 2.0 ** (e - 1) * (1 + 1e-9)
    assert g == int((n.astype(np.int64) ** 2).sum())
    assert q == pytest.approx(np.sqrt(((n.T * 2.0 ** e - y) ** 2).sum() / 50), rel=1e-9)
    assert q <= np.sqrt(3) * 2.0 ** (e - 1)


@pytest.mark.parametrize("L", [5, 47, 300])
def test_fast_and_exact_paths_match_oracle(hooks, oracle_mod, L):
    rng = np.random.default_rng(L)
    base = synth.base_chain(L, rng)
    xs = synth.decoys(base, 14, rng, near_dup_frac=0.25)
    rot = synth.random_rotations(1, rng)[0]
    xs = np.concatenate([xs, np.stack([xs[0].copy(), xs[1] @ rot.T + 3.0, xs[2] + rng.normal(size=(L, 3)) * 1e-4])])
    e = _grid_exp(xs)
    n = xs.shape[0]
    dig = [hooks.digits(x, e) for x in xs]
    flagged = 0
    for i in range(n):
        for j in range(i + 1, n):
            ref = oracle_mod.crmsd(xs[i], xs[j])
            da, ga, qa = dig[i]
            db, gb, qb = dig[j]
            s = hooks.levels(da, db)
            assert np.abs(s[:3]).max() < 2 ** 24
            r, f = hooks.fast(s, ga, gb, qa, qb, e, L)
            rx = hooks.exact(da, db, e)
            # Minkowski: the quantised pair's crmsd is within qa + qb of the exact one
            assert abs(rx - ref) <= qa + qb + 2e-6, (i, j, rx, ref)
            if f:
                flagged += 1
            else:
                assert abs(r - ref) <= TOL_TOTAL, (i, j, r, ref)
    # exact copies and near-duplicates must be caught by the error bound
    assert flagged >= 1


def test_identical_structures_exact_zero(hooks):
    rng = np.random.default_rng(9)
    x = synth.base_chain(64, rng)
    e = _grid_exp([x])
    d, g, q = hooks.digits(x, e)
    assert hooks.exact(d, d, e) == pytest.approx(0.0, abs=1e-9)
    r, f = hooks.fast(hooks.levels(d, d), g, g, q, q, e, 64)
    assert f == 1 or r <= 1e-4


def _truncated(d, e):
    """The structure the screen's levels 0 and 1 describe (digit 2 dropped):
    its squared norm (grid units) and RMS distance from the full one (A)."""
    n = join(d)
    d2 = d[2] // 16
    t = n - d2
    return float((t.astype(np.float64) ** 2).sum()), float(np.sqrt((d2.astype(np.float64) ** 2).sum() / d.shape[2])
                                                          * 2.0 ** e)


@pytest.mark.parametrize("L", [8, 64, 300])
def test_screen_bracket_contains_crmsd(hooks, oracle_mod, L):
    """The serving screen's Newton bracket (levels 0 and 1 only) contains the
    exact crmsd of the quantised pair, for near, far, identical, mirrored and
    planar pairs; and it is tight for near pairs."""
    rng = np.random.default_rng(100 + L)
    base = synth.base_chain(L, rng)
    xs = list(synth.decoys(base, 10, rng, near_dup_frac=0.3))
    xs.append(xs[0].copy())                                 # identical
    xs.append(xs[1] * np.array([1.0, 1.0, -1.0]))           # mirror image
    flat = rng.normal(size=(L, 3)) * 10.0
    flat[:, 2] = 0.0
    xs.append(flat)                                          # planar
    xs.append(synth.base_chain(L, rng))                      # unrelated chain
    xs = np.stack(xs)
    e = _grid_exp(xs)
    dig = [hooks.digits(x, e) for x in xs]
    tr = [_truncated(d[0], e) for d in dig]
    fp = ctypes.POINTER(ctypes.c_float)
    widths = []
    for i in range(len(xs)):
        for j in range(i + 1, len(xs)):
            da, ga, qa = dig[i]
            db, gb, qb = dig[j]
            s = hooks.levels(da, db)
            s11 = np.array([[(da[1, x] * db[1, y]).sum() for y in range(3)] for x in range(3)], dtype=np.float64)
            m9 = np.ascontiguousarray((s[0] + s[1] / 512.0 + s11 / 2.0 ** 18).reshape(9), dtype=np.float32)
            lo, hi = ctypes.c_float(), ctypes.c_float()
            st = hooks.lib.bs_selftest_screen(m9.ctypes.data_as(fp), tr[i][0] + tr[j][0], 0.0, tr[i][1] + tr[j][1], e,
                                              L, ctypes.byref(lo), ctypes.byref(hi))
            assert st == 0
            rx = hooks.exact(da, db, e)
            assert lo.value <= rx * (1 + 1e-6) + 1e-9 and rx <= hi.value * (1 + 1e-6) + 1e-9, (i, j, lo.value, rx,
                                                                                                 hi.value)
            ref = oracle_mod.crmsd(xs[i], xs[j])
            assert lo.value - (qa + qb) - 1e-6 <= ref <= hi.value + qa + qb + 1e-6
            if 0.5 < rx < 5.0:
                # the bracket's width in E / L = 2 r dr, relative to (Ga + Gb) / L
                widths.append(2 * (hi.value - lo.value) * rx / ((tr[i][0] + tr[j][0]) * 2.0 ** (2 * e) / L))
    # near pairs of protein-sized chains: the proven error bound of the FP32
    # quartic (2^-16 on P and P') fixes the top root to ~2^-13 of (Ga + Gb);
    # short chains are elongated, their top root nearly double: wider
    if L >= 64:
        assert max(widths) < 2.5e-4, max(widths)
