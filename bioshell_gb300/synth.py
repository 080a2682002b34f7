"""Seeded synthetic decoy sets for the crmsd workloads.

The reference has no crmsd benchmark data, so every workload is generated:

* a base chain: CA-only random self-avoiding chain of ``L`` residues with
  3.8 A virtual bonds, planar angles uniform in [80, 150] degrees and
  dihedrals uniform in [-180, 180) degrees, built by natural-extension
  reference-frame placement; a step is redrawn when the new atom comes closer
  than 3.8 A to any non-adjacent atom already placed;
* decoys: base + iid Gaussian noise N(0, sigma^2) per coordinate, sigma drawn
  per decoy, followed by a uniformly random rotation (normalised 4-D Gaussian
  quaternion) and a translation uniform in [-50, 50]^3 A;
* optional near-duplicates: a random subset of decoys whose noise is a fixed
  small sigma (stresses the cancellation step).

All coordinates are float64 AoS ``[n][L][3]``, the layout of
``bioshell_core::Vec3`` triples (bioshell-core/src/vec3.rs:44-51).
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

BOND = 3.8


def base_chain(L: int, rng: np.random.Generator, max_restarts: int = 200) -> np.ndarray:
    """Random self-avoiding CA chain, [L][3] float64."""
    if L < 1:
        raise ValueError("L must be >= 1")
    for _ in range(max_restarts):
        pts = np.zeros((L, 3))
        if L == 1:
            return pts
        pts[1] = (BOND, 0.0, 0.0)
        if L > 2:
            th = math.radians(rng.uniform(80.0, 150.0))
            pts[2] = pts[1] + BOND * np.array([-math.cos(th), math.sin(th), 0.0])
        ok = True
        for i in range(3, L):
            a, b, c = pts[i - 3], pts[i - 2], pts[i - 1]
            bc = c - b
            bc /= np.linalg.norm(bc)
            nrm = np.cross(b - a, bc)
            nrm /= np.linalg.norm(nrm)
            m = np.cross(nrm, bc)
            placed = False
            for _try in range(100):
                th = math.radians(rng.uniform(80.0, 150.0))
                ph = math.radians(rng.uniform(-180.0, 180.0))
                d = np.array([-BOND * math.cos(th), BOND * math.sin(th) * math.cos(ph),
                              BOND * math.sin(th) * math.sin(ph)])
                p = c + d[0] * bc + d[1] * m + d[2] * nrm
                # non-adjacent atoms: every placed atom except the predecessor
                d2 = np.sum((pts[: i - 1] - p) ** 2, axis=1)
                if np.all(d2 >= BOND * BOND):
                    pts[i] = p
                    placed = True
                    break
            if not placed:
                ok = False
                break
        if ok:
            return pts
    raise RuntimeError(f"could not grow a self-avoiding chain of length {L}")


def random_rotations(n: int, rng: np.random.Generator) -> np.ndarray:
    """n uniformly random proper rotations, [n][3][3]."""
    q = rng.normal(size=(n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    w, x, y, z = q.T
    r = np.empty((n, 3, 3))
    r[:, 0, 0] = w * w + x * x - y * y - z * z
    r[:, 0, 1] = 2 * (x * y - w * z)
    r[:, 0, 2] = 2 * (x * z + w * y)
    r[:, 1, 0] = 2 * (x * y + w * z)
    r[:, 1, 1] = w * w - x * x + y * y - z * z
    r[:, 1, 2] = 2 * (y * z - w * x)
    r[:, 2, 0] = 2 * (x * z - w * y)
    r[:, 2, 1] = 2 * (y * z + w * x)
    r[:, 2, 2] = w * w - x * x - y * y + z * z
    return r


def decoys(base: np.ndarray, n: int, rng: np.random.Generator, sigma=(0.5, 4.0),
           near_dup_frac: float = 0.0, near_dup_sigma: float = 0.01,
           chunk: int = 8192, return_sigma: bool = False):
    """n noisy, randomly placed copies of ``base`` -> [n][L][3] float64
    (and the per-decoy noise sigma when ``return_sigma``)."""
    L = base.shape[0]
    sig = rng.uniform(sigma[0], sigma[1], size=n)
    if near_dup_frac > 0.0:
        k = int(round(near_dup_frac * n))
        idx = rng.choice(n, size=k, replace=False)
        sig[idx] = near_dup_sigma
    out = np.empty((n, L, 3))
    for s in range(0, n, chunk):
        e = min(n, s + chunk)
        m = e - s
        noisy = base[None, :, :] + rng.normal(size=(m, L, 3)) * sig[s:e, None, None]
        rot = random_rotations(m, rng)
        shift = rng.uniform(-50.0, 50.0, size=(m, 1, 3))
        out[s:e] = np.einsum("nkj,nij->nki", noisy, rot) + shift
    return (out, sig) if return_sigma else out


@dataclass(frozen=True)
class Workload:
    name: str
    n: int
    L: int
    sigma: tuple = (0.5, 4.0)
    near_dup_frac: float = 0.0
    near_dup_sigma: float = 0.01
    seed: int = 0

    @property
    def pairs(self) -> int:
        return self.n * (self.n - 1) // 2

    def generate(self, return_sigma: bool = False):
        rng = np.random.Generator(np.random.PCG64(self.seed))
        base = base_chain(self.L, rng)
        return decoys(base, self.n, rng, self.sigma, self.near_dup_frac, self.near_dup_sigma,
                      return_sigma=return_sigma)


# The workloads the crmsd engine is measured on (sizes from the project spec).
PLAIN_CPU = Workload("decoys-500x64", n=500, L=64, seed=0)
PLAIN_FP64_GPU = Workload("decoys-20000x150", n=20000, L=150, seed=1)
MIXED_50K = Workload("decoys-50000x300-neardup5", n=50000, L=300, near_dup_frac=0.05,
                     near_dup_sigma=0.01, seed=2)


def batched_sets(nsets: int = 256, seed: int = 3, n_range=(50, 4000), l_range=(40, 800),
                 sigma=(0.2, 6.0)):
    """Independent decoy sets with log-uniform sizes and chain lengths."""
    rng = np.random.Generator(np.random.PCG64(seed))
    sets = []
    for _ in range(nsets):
        n = int(round(math.exp(rng.uniform(math.log(n_range[0]), math.log(n_range[1])))))
        L = int(round(math.exp(rng.uniform(math.log(l_range[0]), math.log(l_range[1])))))
        base = base_chain(L, rng)
        sets.append(decoys(base, n, rng, sigma))
    return sets


# The serving workload: a library bucketed by chain length with shares that
# total ~1.7e7 atoms for 200,000 structures (85/9/4/2% at L = 64/128/256/512),
# each bucket made of decoy families around independent base chains.
SERVING_BUCKETS = ((64, 0.85), (128, 0.09), (256, 0.04), (512, 0.02))


def serving_library(n_total: int = 200_000, families: int = 32, seed: int = 4, sigma=(0.5, 4.0)):
    """{L: [n_L][L][3] decoys} and {L: [families] base chains (centred)}."""
    rng = np.random.Generator(np.random.PCG64(seed))
    lib, bases = {}, {}
    for L, share in SERVING_BUCKETS:
        n = int(round(n_total * share))
        fb = [base_chain(L, rng) for _ in range(families)]
        fb = [b - b.mean(axis=0) for b in fb]
        per = [n // families + (1 if f < n % families else 0) for f in range(families)]
        lib[L] = np.concatenate([decoys(fb[f], per[f], rng, sigma) for f in range(families)])
        bases[L] = fb
    return lib, bases


def serving_queries(bases, pool: int = 1024, seed: int = 5, sigma=(0.5, 4.0)):
    """A pool of query decoys per bucket (contiguous slices are the requests)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    out = {}
    for L, fb in bases.items():
        fam = rng.integers(len(fb), size=pool)
        out[L] = np.concatenate([decoys(fb[f], 1, rng, sigma) for f in fam])
    return out
