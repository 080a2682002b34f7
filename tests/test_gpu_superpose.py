"""bs_superpose / bs_superpose_pairs on the GPU: the rototranslation of each
pair against the SVD-Kabsch oracle and the host copy of the same math, the
RMSD against the QCP crmsd oracle, device pointers, and the error paths."""
import ctypes

import numpy as np
import pytest

from bioshell_gb300 import CrmsdError, synth

pytestmark = pytest.mark.gpu


def host_superpose(lib, a, b):
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    rot, t, r = np.empty(9), np.empty(3), ctypes.c_double()
    assert lib.bs_selftest_superpose(a.ctypes.data, b.ctypes.data, a.shape[0], rot.ctypes.data, t.ctypes.data,
                                     ctypes.byref(r)) == 0
    return rot.reshape(3, 3), t, r.value


@pytest.mark.parametrize("L", [5, 64, 300, 777])
def test_superpose_pairs_match_oracles(engine, enginelib, oracle_mod, L):
    rng = np.random.default_rng(500 + L)
    base = synth.base_chain(L, rng)
    xs = synth.decoys(base, 40, rng, near_dup_frac=0.2)
    ii = rng.integers(0, 40, 300)
    jj = rng.integers(0, 40, 300)
    rot, trans, rmsd = engine.superpose_pairs(xs, ii, jj)
    for t in range(len(ii)):
        i, j = ii[t], jj[t]
        rk, tk, rr = oracle_mod.kabsch_superpose(xs[i], xs[j])
        assert abs(rmsd[t] - rr) <= 1e-9 * max(1.0, rr), (t, rmsd[t], rr)
        # the QCP oracle forms E = G_a + G_b - 2 lambda: near E = 0 its RMSD
        # carries the cancellation, ~sqrt(1e-16 G / L) (1.5e-7 A for i == j)
        g = sum(((x - x.mean(0)) ** 2).sum() for x in (xs[i], xs[j]))
        floor = np.sqrt(1e-14 * g / L)
        assert abs(rmsd[t] - oracle_mod.crmsd(xs[i], xs[j])) <= 1e-8 * max(1.0, rr) + floor
        np.testing.assert_allclose(rot[t] @ rot[t].T, np.eye(3), atol=1e-12)
        assert abs(np.linalg.det(rot[t]) - 1.0) < 1e-12
        if i != j:
            np.testing.assert_allclose(rot[t], rk, atol=1e-8)
            np.testing.assert_allclose(trans[t], tk, atol=1e-6)
        hr, ht, hrm = host_superpose(enginelib, xs[i], xs[j])
        np.testing.assert_allclose(rot[t], hr, atol=1e-11)
        assert abs(rmsd[t] - hrm) <= 1e-11 * max(1.0, hrm)
        res = xs[j] @ rot[t].T + trans[t] - xs[i]
        assert abs(np.sqrt((res * res).sum() / L) - rmsd[t]) <= 1e-11 * max(1.0, rr)


def test_superpose_single_pair_and_device_pointers(engine, oracle_mod):
    import torch

    rng = np.random.default_rng(8)
    a = synth.base_chain(120, rng)
    b = synth.decoys(a, 1, rng)[0]
    rt, r = engine.superpose(a, b)
    rk, tk, rr = oracle_mod.kabsch_superpose(a, b)
    np.testing.assert_allclose(rt.rotation(), rk, atol=1e-9)
    np.testing.assert_allclose(rt.translation(), tk, atol=1e-7)
    assert abs(r - rr) <= 1e-9 * max(1.0, rr)
    np.testing.assert_allclose(rt.apply(b), a, atol=3 * r + 1e-9)
    # device coordinates and outputs
    xs = torch.from_numpy(np.stack([a, b])).cuda()
    ii = torch.tensor([0, 1], dtype=torch.int64, device="cuda")
    jj = torch.tensor([1, 0], dtype=torch.int64, device="cuda")
    rot = torch.empty((2, 3, 3), dtype=torch.float64, device="cuda")
    trans = torch.empty((2, 3), dtype=torch.float64, device="cuda")
    rm = torch.empty(2, dtype=torch.float64, device="cuda")
    lib = engine._lib
    assert lib.bs_superpose_pairs(engine._h, xs.data_ptr(), 2, 120, ii.data_ptr(), jj.data_ptr(), 2, rot.data_ptr(),
                                  trans.data_ptr(), rm.data_ptr()) == 0
    torch.cuda.synchronize()
    np.testing.assert_allclose(rot[0].cpu().numpy(), rk, atol=1e-9)
    assert abs(rm[0].item() - rr) <= 1e-9 * max(1.0, rr)
    assert abs(rm[1].item() - rr) <= 1e-9 * max(1.0, rr)
    # the reverse superposition is the inverse transform
    np.testing.assert_allclose(rot[1].cpu().numpy(), rk.T, atol=1e-9)


def test_superpose_errors(engine):
    rng = np.random.default_rng(2)
    xs = rng.normal(size=(4, 10, 3))
    with pytest.raises(CrmsdError):
        engine.superpose_pairs(xs, [0, 4], [1, 2])
    bad = xs.copy()
    bad[2, 3, 1] = np.nan
    with pytest.raises(CrmsdError):
        engine.superpose_pairs(bad, [0, 2], [1, 3])
    # the context stays usable
    rot, trans, rmsd = engine.superpose_pairs(xs, [0], [1])
    assert np.isfinite(rmsd).all()
    rot, trans, rmsd = engine.superpose_pairs(xs, [], [])
    assert rot.shape == (0, 3, 3)
