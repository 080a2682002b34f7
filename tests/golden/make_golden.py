"""Regenerates the committed golden fixtures of the crmsd tests.

    BIOSHELL_REFERENCE=path/to/reference/checkout python tests/golden/make_golden.py

* ``decoys_small.npz``   -- a seeded decoy set (32 x 47 atoms, including
  near-duplicates, an exact copy and a rigidly moved copy) with the FP64 QCP
  oracle's packed triangle and the independent SVD-Kabsch triangle;
* ``models_2jqb.npz``    -- the 20 NMR models of PDB entry 2JQB read from the
  reference's own multi-model fixture bioshell-pdb/tests/test_files/2jqb.cif
  (the file bioshell-pdb/tests/test_structure.rs:155-166 loads), all 255 atoms
  and the CA subset, with oracle triangles for both;
* ``hierarchical_reference_tests.json`` -- the inputs and expected outputs of
  bioshell-clustering/tests/test_hierarchical.rs:10-71, read from the test
  source and the d5.tsv fixture it uses.

The reference checkout (named by the BIOSHELL_REFERENCE environment variable,
or the first argument) is needed for the last two; the script is run once on
a machine that has it, and its outputs are committed.  Without it, only
the first fixture is regenerated and the script says so.
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from bioshell_gb300 import synth  # noqa: E402
from oracle import oracle  # noqa: E402


def small_decoys():
    rng = np.random.Generator(np.random.PCG64(20240601))
    base = synth.base_chain(47, rng)
    x = synth.decoys(base, 29, rng, sigma=(0.3, 3.0), near_dup_frac=0.15, near_dup_sigma=0.01)
    rot = synth.random_rotations(1, rng)[0]
    extra = np.stack([x[3].copy(), x[5] @ rot.T + np.array([7.0, -3.0, 11.0]), x[7] + rng.normal(size=x[7].shape) * 1e-3])
    x = np.concatenate([x, extra])
    n = x.shape[0]
    ii, jj = np.triu_indices(n, 1)
    tri = oracle.crmsd_all_vs_all(x, nthreads=1)
    svd = oracle.kabsch_pairs(x, ii, jj)
    np.savez_compressed(os.path.join(HERE, "decoys_small.npz"), xyz=x, rmsd=tri, rmsd_svd=svd)


def parse_2jqb(path):
    models_all, models_ca = {}, {}
    in_loop = False
    cols = []
    with open(path) as fh:
        for line in fh:
            if line.startswith("_atom_site."):
                in_loop = True
                cols.append(line.strip().split(".", 1)[1])
                continue
            if in_loop and (line.startswith("ATOM") or line.startswith("HETATM")):
                f = line.split()
                rec = dict(zip(cols, f))
                m = int(rec["pdbx_PDB_model_num"])
                xyz = (float(rec["Cartn_x"]), float(rec["Cartn_y"]), float(rec["Cartn_z"]))
                models_all.setdefault(m, []).append(xyz)
                if rec["label_atom_id"] == "CA":
                    models_ca.setdefault(m, []).append(xyz)
            elif in_loop and cols and line.startswith("#"):
                in_loop = False
    keys = sorted(models_all)
    return np.array([models_all[k] for k in keys]), np.array([models_ca[k] for k in keys])


def models_2jqb(ref):
    path = os.path.join(ref, "bioshell-pdb", "tests", "test_files", "2jqb.cif")
    allat, ca = parse_2jqb(path)
    np.savez_compressed(os.path.join(HERE, "models_2jqb.npz"), all_atoms=allat, ca=ca,
                        rmsd_all=oracle.crmsd_all_vs_all(allat, nthreads=1),
                        rmsd_ca=oracle.crmsd_all_vs_all(ca, nthreads=1))


def hierarchical_tests(ref):
    tsv = os.path.join(ref, "bioshell-clustering", "tests", "test_files", "d5.tsv")
    rows = []
    with open(tsv) as fh:
        for line in fh:
            a, b, v = line.split()
            rows.append([a, b, float(v)])
    out = {
        "source": "bioshell-clustering/tests/test_hierarchical.rs:10-71",
        "cluster_numbers": {"data": [6.0, 2.0, 2.5, 5.9], "rule": "single_link",
                            "order": [6.0, 5.9, 2.0, 2.5], "order_balanced": [6.0, 5.9, 2.5, 2.0]},
        "cluster_letters": {"data": list("AZDYCXBWFV"), "rule": "single_link",
                            "order": list("ABDCFZYXWV"), "order_balanced": list("ABCDFVWXYZ")},
        "cluster_distance_matrix": {"tsv": rows, "rule": "single_link", "cutoff": 0.11, "n_clusters": 4,
                                    "n_points": 5, "largest": 2},
    }
    with open(os.path.join(HERE, "hierarchical_reference_tests.json"), "w") as fh:
        json.dump(out, fh, indent=1)


if __name__ == "__main__":
    oracle.build()
    small_decoys()
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("BIOSHELL_REFERENCE", "")
    if ref and os.path.isdir(ref):
        models_2jqb(ref)
        hierarchical_tests(ref)
    else:
        print("BIOSHELL_REFERENCE names no reference checkout: only decoys_small.npz was regenerated")
    print("golden fixtures written to", HERE)
