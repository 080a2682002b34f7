"""The synthetic workload generator follows its stated specification."""
import numpy as np

from bioshell_gb300 import synth


def test_base_chain_geometry():
    rng = np.random.default_rng(0)
    x = synth.base_chain(120, rng)
    bonds = np.linalg.norm(np.diff(x, axis=0), axis=1)
    np.testing.assert_allclose(bonds, 3.8, atol=1e-9)
    v1, v2 = x[:-2] - x[1:-1], x[2:] - x[1:-1]
    ang = np.degrees(np.arccos(np.sum(v1 * v2, 1) / (np.linalg.norm(v1, axis=1) * np.linalg.norm(v2, axis=1))))
    assert ang.min() >= 80.0 - 1e-6 and ang.max() <= 150.0 + 1e-6
    d = np.linalg.norm(x[:, None] - x[None], axis=2)
    nonadj = np.abs(np.arange(120)[:, None] - np.arange(120)[None]) >= 2
    assert d[nonadj].min() >= 3.8 - 1e-9


def test_rotations_are_proper():
    r = synth.random_rotations(100, np.random.default_rng(1))
    np.testing.assert_allclose(np.einsum("nij,nkj->nik", r, r), np.broadcast_to(np.eye(3), (100, 3, 3)), atol=1e-12)
    np.testing.assert_allclose(np.linalg.det(r), 1.0, atol=1e-12)


def test_workload_shapes_and_determinism():
    w = synth.Workload("t", n=64, L=33, near_dup_frac=0.1, seed=5)
    a, b = w.generate(), w.generate()
    assert a.shape == (64, 33, 3) and a.dtype == np.float64
    np.testing.assert_array_equal(a, b)
    assert synth.MIXED_50K.pairs == 1249975000
    assert synth.PLAIN_CPU.pairs == 124750
