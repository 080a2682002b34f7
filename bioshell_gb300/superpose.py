"""Superposition output: the reference's ``Rototranslation`` and the GPU call
that produces one per pair.

``Rototranslation`` mirrors ``bioshell_pdb::calc::Rototranslation``
(bioshell-pdb/src/calc/transformation.rs): ``new(rot, t)`` stores the
rotation, the translation and the inverse (``:22-37``); ``apply`` maps
v -> R v + t (``apply_mut``, ``:171-174``) and ``apply_inverse`` maps
v -> R^-1 v - R^-1 t; ``set_translation`` updates the inverse translation.
The rotation and translation that superpose one structure on another come
from ``Engine.superpose`` / ``Engine.superpose_pairs`` (``bs_superpose*``).
"""
from __future__ import annotations

import numpy as np


class Rototranslation:
    """Rotation-translation operation in 3D: v -> R v + t."""

    def __init__(self, rot, t):
        self._rotation = np.array(rot, dtype=np.float64).reshape(3, 3)
        self._translation = np.array(t, dtype=np.float64).reshape(3)
        self._inverse_rotation = np.linalg.inv(self._rotation)
        self._inverse_translation = -(self._inverse_rotation @ self._translation)

    @classmethod
    def new(cls, rot, t) -> "Rototranslation":
        return cls(rot, t)

    def rotation(self) -> np.ndarray:
        return self._rotation

    def translation(self) -> np.ndarray:
        return self._translation

    def set_translation(self, t) -> None:
        self._translation = np.array(t, dtype=np.float64).reshape(3)
        self._inverse_translation = -(self._inverse_rotation @ self._translation)

    def apply(self, v) -> np.ndarray:
        """R v + t for one point [3] or many [..., 3]."""
        v = np.asarray(v, dtype=np.float64)
        return v @ self._rotation.T + self._translation

    def apply_inverse(self, v) -> np.ndarray:
        v = np.asarray(v, dtype=np.float64)
        return v @ self._inverse_rotation.T + self._inverse_translation

    def __repr__(self) -> str:
        return f"Rototranslation(rotation={self._rotation.tolist()}, translation={self._translation.tolist()})"
