"""The YAML-in / HDF5-out boundary on the CPU: the YAML subset parser, the
configuration (SpinED.hs:81-173 FromJSON instances, the reference's own
parser test cases in test/Spec.hs) and the HDF5 writer/reader round trip."""
import glob
import os

import numpy as np
import pytest

from spined import config as CF
from spined import hdf5 as H
from spined import yaml_subset as Y

README_CONFIG = """
basis:
  number_spins: 4
  symmetries: []
hamiltonian:
  name: "Heisenberg Hamiltonian"
  terms:
    - matrix: [[1,  0,  0,  0],
               [0, -1,  2,  0],
               [0,  2, -1,  0],
               [0,  0,  0,  1]]
      sites: [[0, 1], [1, 2], [2, 3], [3, 0]]
observables: []
"""


def test_yaml_scalars_and_collections():
    v = Y.loads("a: [1, -2, 2.5e-3, .5, 'it''s', \"x # y\", null, ~, true]\n"
                "b:\n  - 1\n  - {c: d, e: [f, 'g']}\n  -\n    h: 3\n"
                "c: plain text  # comment\n"
                "d: [ [1, [2, 3]],\n     [4, 5] ]\n"
                "e:\n- x\n- y\n")
    assert v == {"a": [1, -2, 0.0025, 0.5, "it's", "x # y", None, None, True],
                 "b": [1, {"c": "d", "e": ["f", "g"]}, {"h": 3}],
                 "c": "plain text", "d": [[1, [2, 3]], [4, 5]], "e": ["x", "y"]}


@pytest.mark.parametrize("bad", ["a: &x 1", "a: |\n  text", "a: [1, 2", "a: 1\n  b: 2", "a: 1\na: 2"])
def test_yaml_rejects_unsupported(bad):
    with pytest.raises(Y.YamlError):
        Y.loads(bad)


def test_symmetry_spec_cases_of_the_reference_tests():
    # test/Spec.hs:22-40 ("flip" is an extra key there, ignored here)
    s = CF.parse_symmetry(Y.loads("permutation: [3, 1, 2, 4]\nflip: true\nsector: 8"))
    assert (s.permutation, s.sector) == ([3, 1, 2, 4], 8)
    s = CF.parse_symmetry(Y.loads("permutation: [1, 1, 2, 4]\nsector: -5"))
    assert (s.permutation, s.sector) == ([1, 1, 2, 4], -5)


def test_basis_spec_cases_of_the_reference_tests():
    # test/Spec.hs:55-87
    b = CF.parse_basis(Y.loads("number_spins: 4\nhamming_weight: 2\nsymmetries:\n"
                               "  - permutation: [1, 2, 3, 0]\n    sector: 0\n"
                               "  - permutation: [3, 2, 1, 0]\n    sector: 0"))
    assert b.number_spins == 4 and b.hamming_weight == 2 and b.spin_inversion is None
    assert [s.permutation for s in b.symmetries] == [[1, 2, 3, 0], [3, 2, 1, 0]]
    b = CF.parse_basis(Y.loads("number_spins: 100\nhamming_weight: null\nsymmetries: []"))
    assert b.number_spins == 100 and b.hamming_weight is None and b.symmetries == []


def test_readme_config_and_defaults():
    c = CF.loads_config(README_CONFIG)
    assert c.output == "exact_diagonalization_result.h5" and c.number_vectors == 1
    assert c.precision == 0.0 and c.datatype == "float64"
    assert c.hamiltonian.terms[0].matrix[1][2] == 2 and len(c.hamiltonian.terms[0].sites) == 4


def test_complex_entries_and_errors():
    c = CF.loads_config(README_CONFIG.replace("[0, -1,  2,  0]", "[0, -1, [2, 0.5], 0]"))
    assert c.hamiltonian.terms[0].matrix[1][2] == complex(2, 0.5)
    with pytest.raises(CF.ConfigError, match="Datatype"):
        CF.loads_config(README_CONFIG + "datatype: float16\n")
    with pytest.raises(CF.ConfigError, match="observables"):
        CF.loads_config(README_CONFIG.replace("observables: []", ""))


REF = os.environ.get("SPINED_REFERENCE_DIR", "")


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "example")),
                    reason="SPINED_REFERENCE_DIR does not name the reference tree")
def test_reference_examples_parse():
    files = sorted(glob.glob(os.path.join(REF, "example", "*.yaml")))
    assert files
    for f in files:
        c = CF.read_config(f)
        n = c.basis.number_spins
        for s in c.basis.symmetries:
            assert sorted(s.permutation) == list(range(n)), f
        for t in c.hamiltonian.terms:
            k = len(t.sites[0])
            assert len(t.matrix) == 2 ** k and all(len(r) == 2 ** k for r in t.matrix), f


def _tree():
    rng = np.random.default_rng(0)
    root = H.Group()
    root.require("/basis")["representatives"] = np.arange(100, dtype=np.uint64) * 7
    h = root.require("hamiltonian")
    h["eigenvalues"] = np.array([-8.0, -4.0])
    h["eigenvectors"] = rng.normal(size=(2, 37))
    h["residuals"] = np.array([1e-10, 3e-9])
    o = root.require("observables")
    for k in range(21):  # more names than one symbol-table node holds
        o[f"O{k:02d}"] = (rng.normal(size=2) + 1j * rng.normal(size=2))
    root.require("_workspace")
    root["vec32"] = rng.normal(size=(3, 5)).astype(np.float32)
    root["cvec64"] = (rng.normal(size=4) + 1j).astype(np.complex64)
    root["ints"] = np.array([-3, 4], dtype=np.int32)
    return root


def _same(a, b):
    if isinstance(a, dict):
        assert isinstance(b, dict) and sorted(a) == sorted(b)
        for k in a:
            _same(a[k], b[k])
    else:
        assert a.dtype == b.dtype and a.shape == b.shape and np.array_equal(a, b)


def test_hdf5_round_trip(tmp_path):
    p = str(tmp_path / "r.h5")
    root = _tree()
    H.write(p, root)
    with open(p, "rb") as f:
        head = f.read(16)
    assert head[:8] == b"\x89HDF\r\n\x1a\n" and head[8] == 0  # superblock version 0
    _same(root, H.read(p))
    # rewrite with an overwritten dataset (the reference's writeDataset)
    r2 = H.read(p)
    r2["hamiltonian"]["eigenvalues"] = np.array([-9.0])
    H.write(p, r2)
    assert H.read(p)["hamiltonian"]["eigenvalues"].tolist() == [-9.0]


def test_hdf5_layout_details(tmp_path):
    """Structures a libhdf5 reader checks: 8-byte alignment of every object,
    the local heap's free block, full-size B-tree and symbol-table nodes."""
    p = str(tmp_path / "d.h5")
    H.write(p, _tree())
    data = open(p, "rb").read()
    assert len(data) % 8 == 0
    for sig, size in ((b"TREE", 24 + 65 * 8), (b"SNOD", 8 + 8 * 40)):
        pos = data.find(sig)
        while pos >= 0:
            assert pos % 8 == 0 and pos + size <= len(data)
            pos = data.find(sig, pos + 1)
    import struct
    pos = data.find(b"HEAP")
    while pos >= 0:
        size, free, addr = struct.unpack_from("<QQQ", data, pos + 8)
        assert free < size and addr % 8 == 0 and size % 8 == 0
        nxt, fsize = struct.unpack_from("<QQ", data, addr + free)
        assert nxt == 1 and fsize == size - free
        pos = data.find(b"HEAP", pos + 1)


def test_hdf5_rejects_garbage(tmp_path):
    p = tmp_path / "x.h5"
    p.write_bytes(b"not hdf5 at all")
    with pytest.raises(H.H5Error):
        H.read(str(p))


def test_square_patches_are_translation_covariant():
    """The patch table of the size-independent network (spined/lattices.py):
    row i lists the (2r+1)^2 sites around site i in a fixed offset order, so
    translating the lattice translates every patch; the same offsets on any L."""
    from spined import lattices as LT
    for L in (4, 6):
        P = LT.square_patches(L)
        assert P.shape == (L * L, 9) and P.dtype == np.uint16
        tx = LT.square_symmetries(L)[0]  # x -> x + 1
        for i in range(L * L):
            assert P[i, 4] == i  # the centre
            assert sorted(set(P[i].tolist())) == sorted(P[i].tolist())  # nine distinct sites
            assert [tx[s] for s in P[i]] == P[tx[i]].tolist()
    # the offsets are the same on both sizes: (dx, dy) of column k
    for L in (4, 6):
        P = LT.square_patches(L)
        off = [(int(s) % L, int(s) // L) for s in P[0]]  # (x, y) of the patch of site (0, 0)
        assert off == [(dx % L, dy % L) for dy in (-1, 0, 1) for dx in (-1, 0, 1)]


def test_j1j2_chain_workload_is_seeded():
    """The batched workload (128 J1-J2 chains): deterministic for a seed, N even in 16..28,
    J2/J1 in [0, 0.6], and the sublattice mask of a ring marks every other site."""
    from spined import lattices as LT
    a = LT.j1j2_chains(128, seed=2024)
    b = LT.j1j2_chains(128, seed=2024)
    assert [(m.number_spins, m.meta["j2"]) for m in a] == [(m.number_spins, m.meta["j2"]) for m in b]
    assert all(m.number_spins % 2 == 0 and 16 <= m.number_spins <= 28 for m in a)
    assert all(0.0 <= m.meta["j2"] <= 0.6 for m in a)
    assert {m.number_spins for m in a} == set(range(16, 29, 2))
    assert LT.chain_sublattice_mask(6) == 0b010101
    assert bin(LT.square_sublattice_mask(4)).count("1") == 8
