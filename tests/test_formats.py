"""The data formats either side of the path (host code, no GPU needed):

* multi-model ingestion (bs_models_*): PDB and mmCIF files written here from
  the committed 2JQB ensemble (20 models x 255 atoms) read back exactly, with
  the reference's CA selection rules (" CA " names; calcium is not CA);
  the reference's own 2jqb.cif when BIOSHELL_REFERENCE names a checkout;
* distance-matrix TSV (bs_tsv_*): the reference's d5.tsv vectors through the
  reader and the hierarchical clustering, printf-exact formatting, round
  trips.
"""
import json
import os

import numpy as np
import pytest

from bioshell_gb300 import clustering as K
from bioshell_gb300 import formats as F

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")
NAMES = [" N  ", " CA ", " C  ", " O  ", " CB "]
ELEMS = ["N", "C", "C", "O", "C"]


def _ensemble():
    z = np.load(os.path.join(GOLD, "models_2jqb.npz"))
    return np.round(z["all_atoms"], 3)


def _write_pdb(path, xyz, calcium=True):
    n, L, _ = xyz.shape
    with open(path, "w") as fh:
        fh.write("HEADER    TEST\n")
        for m in range(n):
            fh.write(f"MODEL     {m + 1:4d}\n")
            for a in range(L):
                name = NAMES[a % 5]
                x, y, z = xyz[m, a]
                fh.write(f"ATOM  {a + 1:5d} {name} ALA A{a // 5 + 1:4d}    {x:8.3f}{y:8.3f}{z:8.3f}  1.00  0.00"
                         f"           {ELEMS[a % 5]}\n")
            if calcium:
                fh.write(f"HETATM{L + 1:5d} CA    CA A 900    {1.0:8.3f}{2.0:8.3f}{3.0:8.3f}  1.00  0.00"
                         f"          CA\n")
            fh.write("ENDMDL\n")
        fh.write("END\n")


def _write_cif(path, xyz, calcium=True):
    n, L, _ = xyz.shape
    cols = ["group_PDB", "id", "type_symbol", "label_atom_id", "label_alt_id", "label_comp_id", "label_asym_id",
            "label_seq_id", "Cartn_x", "Cartn_y", "Cartn_z", "occupancy", "pdbx_PDB_model_num"]
    with open(path, "w") as fh:
        fh.write("data_TEST\n#\nloop_\n")
        for c in cols:
            fh.write(f"_atom_site.{c}\n")
        k = 0
        for m in range(n):
            for a in range(L):
                k += 1
                x, y, z = xyz[m, a]
                nm = NAMES[a % 5].strip()
                fh.write(f"ATOM {k} {ELEMS[a % 5]} {nm} . ALA A {a // 5 + 1} {x:.3f} {y:.3f} {z:.3f} 1.00 {m + 1}\n")
            if calcium:
                k += 1
                fh.write(f"HETATM {k} CA CA . CA B . 1.000 2.000 3.000 1.00 {m + 1}\n")
        fh.write("#\n")


@pytest.mark.parametrize("fmt", ["pdb", "cif"])
def test_models_read_back_exactly(enginelib, tmp_path, fmt):
    xyz = _ensemble()
    p = str(tmp_path / f"ens.{fmt}")
    (_write_pdb if fmt == "pdb" else _write_cif)(p, xyz)
    got = F.read_models(p)  # format detected from the first line
    assert got.shape == (xyz.shape[0], xyz.shape[1] + 1, 3)
    np.testing.assert_array_equal(got[:, :-1], xyz)
    ca = F.read_models(p, ca_only=True)
    np.testing.assert_array_equal(ca, xyz[:, 1::5])  # calcium ions are not alpha carbons


def test_models_errors(enginelib, tmp_path):
    xyz = _ensemble()[:3]
    p = str(tmp_path / "bad.pdb")
    _write_pdb(p, xyz, calcium=False)
    lines = open(p).read().splitlines()
    # drop one atom of the second model: models differ in size
    k = [i for i, l in enumerate(lines) if l.startswith("MODEL")][1] + 3
    open(p, "w").write("\n".join(lines[:k] + lines[k + 1:]) + "\n")
    with pytest.raises(F.FormatError) as e:
        F.read_models(p)
    assert e.value.status == 1
    with pytest.raises(F.FormatError):
        F.read_models(str(tmp_path / "missing.pdb"))


def test_reference_2jqb_when_present(enginelib):
    """With BIOSHELL_REFERENCE pointing at a reference checkout: its own
    2jqb.cif (bioshell-pdb/tests/test_files) read by the engine equals the
    committed fixture made from it."""
    root = os.environ.get("BIOSHELL_REFERENCE")
    ref = os.path.join(root, "bioshell-pdb", "tests", "test_files", "2jqb.cif") if root else ""
    if not ref or not os.path.exists(ref):
        pytest.skip("BIOSHELL_REFERENCE not set to a reference checkout")
    z = np.load(os.path.join(GOLD, "models_2jqb.npz"))
    np.testing.assert_array_equal(F.read_models(ref), z["all_atoms"])
    np.testing.assert_array_equal(F.read_models(ref, ca_only=True), z["ca"])


def test_tsv_reference_vectors(enginelib, tmp_path):
    d5 = json.load(open(os.path.join(GOLD, "hierarchical_reference_tests.json")))["cluster_distance_matrix"]
    p = str(tmp_path / "d5.tsv")
    with open(p, "w") as fh:
        for a, b, v in d5["tsv"]:
            fh.write(f"{a}\t{b}\t{v:.6f}\n")
    labels, m = F.read_tsv(p, default=100.0, symmetric=True)
    assert labels == ["4HGI:A", "6A18:A", "6C3J:A", "7YDL:A", "2NNH:A"]
    for a, b, v in d5["tsv"]:
        assert m.get(labels.index(a), labels.index(b)) == float(np.float32(v))
    tree = K.hierarchical_clustering(m, "single")
    sizes = sorted(np.bincount(K.cut_tree(tree, d5["cutoff"])))
    assert len(sizes) == d5["n_clusters"] and sizes[-1] == d5["largest"] and sum(sizes) == d5["n_points"]
    # read as non-symmetric, lines (j, i) with j after i in label order are not used
    _, m2 = F.read_tsv(p, default=100.0, symmetric=False)
    assert m2.get(0, 4) == 100.0 and m2.get(0, 1) == float(np.float32(0.126))


@pytest.mark.parametrize("dtype,dec", [(np.float64, 6), (np.float32, 3), (np.float64, 9)])
def test_tsv_write_matches_printf(enginelib, tmp_path, dtype, dec):
    rng = np.random.default_rng(3)
    n = 61
    tri = (rng.random(n * (n - 1) // 2) * 40).astype(dtype)
    tri[:7] = [0.0, 0.5, 1e-7, 2.5e-4, 123.4565, 0.0015, 1.0 / 3]  # ties, tiny values
    labels = [f"m{i}:A" for i in range(n)]
    p = str(tmp_path / "out.tsv")
    F.write_tsv(p, tri, labels, decimals=dec, n=n)
    want = []
    k = 0
    for i in range(n):
        for j in range(i + 1, n):
            want.append(f"{labels[i]}\t{labels[j]}\t{float(tri[k]):.{dec}f}")
            k += 1
    assert open(p).read().splitlines() == want
    labs, m = F.read_tsv(p)
    assert labs == labels
    np.testing.assert_array_equal(m.values, np.array([float(f"{float(v):.{dec}f}") for v in tri], dtype=np.float32))
