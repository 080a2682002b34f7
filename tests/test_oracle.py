"""Pins the CPU FP64 oracle (QCP) before anything is compared against it.

The reference has no crmsd routine or golden crmsd values
(bioshell-pdb/src/calc/mod.rs:1-10), so the oracle is pinned by analytic
known answers, by an independent SVD-Kabsch, by numpy's symmetric
eigensolver for the quartic root, and by the committed golden fixtures --
including the reference's own multi-model ensemble 2jqb.cif
(bioshell-pdb/tests/test_structure.rs:155-166).
"""
import numpy as np
import pytest

from bioshell_gb300 import synth


def _rot(seed):
    return synth.random_rotations(1, np.random.default_rng(seed))[0]


def test_identity_is_zero(oracle_mod):
    x = synth.base_chain(30, np.random.default_rng(0))
    assert oracle_mod.crmsd(x, x) == 0.0


@pytest.mark.parametrize("L", [3, 4, 17, 64, 300])
def test_rigid_motion_is_zero(oracle_mod, L):
    rng = np.random.default_rng(L)
    x = synth.base_chain(L, rng) + rng.normal(size=(L, 3))
    y = x @ _rot(L).T + rng.uniform(-50, 50, size=3)
    assert oracle_mod.crmsd(x, y) <= 1e-6
    assert oracle_mod.crmsd(x, y) == pytest.approx(0.0, abs=1e-6)


def test_mirror_image_is_positive(oracle_mod):
    x = synth.base_chain(40, np.random.default_rng(3))
    m = x * np.array([-1.0, 1.0, 1.0])
    # a chiral chain cannot be superposed on its mirror image by a proper rotation
    assert oracle_mod.crmsd(x, m) > 0.5


def test_translation_and_centring(oracle_mod):
    rng = np.random.default_rng(4)
    x = rng.normal(size=(25, 3)) * 5
    y = x + rng.normal(size=(25, 3)) * 0.7
    r0 = oracle_mod.crmsd(x, y)
    assert oracle_mod.crmsd(x + 100.0, y - 40.0) == pytest.approx(r0, abs=1e-9)


def test_symmetry(oracle_mod):
    rng = np.random.default_rng(5)
    x = rng.normal(size=(33, 3)) * 8
    y = x @ _rot(9).T + rng.normal(size=(33, 3))
    assert oracle_mod.crmsd(x, y) == pytest.approx(oracle_mod.crmsd(y, x), abs=1e-10)


def test_qcp_matches_svd_kabsch(oracle_mod):
    x = synth.PLAIN_CPU.generate()
    n = x.shape[0]
    tri = oracle_mod.crmsd_all_vs_all(x)
    ii, jj = np.triu_indices(n, 1)
    svd = oracle_mod.kabsch_pairs(x, ii, jj)
    assert np.abs(tri - svd).max() <= 1e-9


def test_lambda_max_matches_eigvalsh(oracle_mod):
    rng = np.random.default_rng(6)
    for _ in range(20):
        L = int(rng.integers(3, 80))
        a = rng.normal(size=(L, 3)) * rng.uniform(1, 20)
        b = a @ _rot(int(rng.integers(1 << 30))).T + rng.normal(size=(L, 3)) * rng.uniform(0, 5)
        lam, ga, gb, _ = oracle_mod.pair_terms(a, b)
        ac, bc = a - a.mean(0), b - b.mean(0)
        s = ac.T @ bc
        sxx, sxy, sxz, syx, syy, syz, szx, szy, szz = s.ravel()
        k = np.array([[sxx + syy + szz, syz - szy, szx - sxz, sxy - syx],
                      [syz - szy, sxx - syy - szz, sxy + syx, szx + sxz],
                      [szx - sxz, sxy + syx, -sxx + syy - szz, syz + szy],
                      [sxy - syx, szx + sxz, syz + szy, -sxx - syy + szz]])
        assert lam == pytest.approx(np.linalg.eigvalsh(k)[-1], rel=1e-12, abs=1e-9)


def test_golden_small(oracle_mod, golden_small):
    x = golden_small["xyz"]
    tri = oracle_mod.crmsd_all_vs_all(x)
    np.testing.assert_allclose(tri, golden_small["rmsd"], rtol=0, atol=1e-12)
    # independent method: SVD loses ~1e-6 A on exact duplicates (its own
    # rounding); elsewhere the two agree to 1e-9 A
    d = np.abs(tri - golden_small["rmsd_svd"])
    assert d.max() <= 1e-6
    assert d[golden_small["rmsd"] > 0.01].max() <= 1e-9


def test_golden_2jqb(oracle_mod, golden_2jqb):
    for key, rk in (("all_atoms", "rmsd_all"), ("ca", "rmsd_ca")):
        x = golden_2jqb[key]
        assert x.shape[0] == 20
        tri = oracle_mod.crmsd_all_vs_all(x)
        np.testing.assert_allclose(tri, golden_2jqb[rk], rtol=0, atol=1e-12)
        ii, jj = np.triu_indices(20, 1)
        assert np.abs(tri - oracle_mod.kabsch_pairs(x, ii, jj)).max() <= 1e-9
    assert golden_2jqb["all_atoms"].shape == (20, 255, 3)


def test_pairs_matches_triangle(oracle_mod, golden_small):
    x = golden_small["xyz"]
    n = x.shape[0]
    ii, jj = np.triu_indices(n, 1)
    np.testing.assert_allclose(oracle_mod.crmsd_pairs(x, ii, jj), golden_small["rmsd"], atol=1e-12, rtol=0)
    # (i, i): the FP64 cancellation G_a + G_b - 2 lambda leaves a floor of
    # ~sqrt(eps G / L) ~ 1e-6 A for identical structures; reversed pairs agree
    assert np.abs(oracle_mod.crmsd_pairs(x, np.arange(n), np.arange(n))).max() <= 2e-6
    np.testing.assert_allclose(oracle_mod.crmsd_pairs(x, jj, ii), golden_small["rmsd"], atol=1e-10, rtol=0)
