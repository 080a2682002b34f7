"""Superposition output (the reference's Rototranslation): the host copy of
the math bs_superpose runs on the GPU, against the SVD-Kabsch oracle and the
QCP crmsd oracle; and the Python Rototranslation's semantics (apply = R v + t,
apply_inverse its inverse) as transformation.rs defines them."""
import ctypes

import numpy as np
import pytest

from bioshell_gb300 import Rototranslation, synth


def host_superpose(lib, a, b):
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    rot, t, r = np.empty(9), np.empty(3), ctypes.c_double()
    st = lib.bs_selftest_superpose(a.ctypes.data, b.ctypes.data, a.shape[0], rot.ctypes.data, t.ctypes.data,
                                   ctypes.byref(r))
    assert st == 0
    return rot.reshape(3, 3), t, r.value


def check_proper(rot):
    np.testing.assert_allclose(rot @ rot.T, np.eye(3), atol=1e-12)
    assert abs(np.linalg.det(rot) - 1.0) < 1e-12


@pytest.mark.parametrize("L", [8, 64, 300])
def test_superpose_matches_kabsch_and_crmsd(enginelib, oracle_mod, L):
    rng = np.random.default_rng(100 + L)
    base = synth.base_chain(L, rng)
    xs = synth.decoys(base, 12, rng, near_dup_frac=0.25)
    for i in range(len(xs)):
        for j in range(len(xs)):
            if i == j:
                continue
            rot, t, r = host_superpose(enginelib, xs[i], xs[j])
            check_proper(rot)
            rk, tk, rr = oracle_mod.kabsch_superpose(xs[i], xs[j])
            ref = oracle_mod.crmsd(xs[i], xs[j])
            assert abs(r - ref) <= 1e-9 * max(1.0, ref), (i, j, r, ref)
            assert abs(r - rr) <= 1e-9 * max(1.0, ref)
            # the optimal rotation is unique for these generic pairs
            np.testing.assert_allclose(rot, rk, atol=1e-8)
            np.testing.assert_allclose(t, tk, atol=1e-6)
            # the transform reproduces its RMSD
            res = xs[j] @ rot.T + t - xs[i]
            assert abs(np.sqrt((res * res).sum() / L) - r) <= 1e-12 * max(1.0, r)


def test_rigid_motion_is_recovered(enginelib):
    rng = np.random.default_rng(7)
    a = synth.base_chain(50, rng)
    r0 = synth.random_rotations(1, rng)[0]
    t0 = np.array([12.5, -40.0, 3.25])
    b = a @ r0.T + t0  # b = R0 a + t0
    rot, t, r = host_superpose(enginelib, a, b)
    np.testing.assert_allclose(rot, r0.T, atol=1e-12)
    np.testing.assert_allclose(t, -(r0.T @ t0), atol=1e-10)
    assert r < 1e-10


@pytest.mark.parametrize("case", ["one_atom", "two_atoms", "collinear", "planar", "mirror", "identical"])
def test_degenerate_pairs(enginelib, oracle_mod, case):
    rng = np.random.default_rng(11)
    if case == "one_atom":
        a, b = rng.normal(size=(1, 3)), rng.normal(size=(1, 3))
    elif case == "two_atoms":
        a, b = rng.normal(size=(2, 3)) * 5, rng.normal(size=(2, 3)) * 5
    elif case == "collinear":
        s = np.linspace(-10, 10, 9)[:, None]
        a = s * np.array([1.0, 2.0, 0.5])
        b = s * np.array([-0.3, 1.0, 2.0]) + 4.0
    elif case == "planar":
        a = np.c_[rng.normal(size=(20, 2)) * 6, np.zeros(20)]
        b = np.c_[rng.normal(size=(20, 2)) * 6, np.zeros(20)]
    elif case == "mirror":
        a = synth.base_chain(30, rng)
        b = a * np.array([-1.0, 1.0, 1.0])
    else:
        a = synth.base_chain(30, rng)
        b = a.copy()
    rot, t, r = host_superpose(enginelib, a, b)
    check_proper(rot)
    _, _, rk = oracle_mod.kabsch_superpose(a, b)
    # the superposition found is optimal even where the rotation is not unique
    assert abs(r - rk) <= 1e-9 * max(1.0, rk), (case, r, rk)
    # (the QCP oracle's Newton iteration loses digits at a repeated root:
    # two atoms give it 2.5e-7 A too little; SVD and the residual agree)
    assert abs(r - oracle_mod.crmsd(a, b)) <= 1e-6 * max(1.0, rk)
    if case == "identical":
        np.testing.assert_allclose(rot, np.eye(3), atol=1e-12)
        assert r < 1e-12


def test_rototranslation_semantics():
    rng = np.random.default_rng(3)
    r0 = synth.random_rotations(1, rng)[0]
    t0 = np.array([1.0, -2.0, 0.5])
    rt = Rototranslation.new(r0, t0)
    v = rng.normal(size=(7, 3))
    np.testing.assert_allclose(rt.apply(v), v @ r0.T + t0, atol=1e-13)
    np.testing.assert_allclose(rt.apply(v[0]), r0 @ v[0] + t0, atol=1e-13)
    np.testing.assert_allclose(rt.apply_inverse(rt.apply(v)), v, atol=1e-12)
    rt.set_translation([0.0, 0.0, 1.0])
    np.testing.assert_allclose(rt.apply_inverse(rt.apply(v)), v, atol=1e-12)
    np.testing.assert_array_equal(rt.translation(), [0.0, 0.0, 1.0])
    np.testing.assert_array_equal(rt.rotation(), r0)
