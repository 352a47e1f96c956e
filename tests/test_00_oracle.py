"""The CPU oracle against every pin the reference holds (README.md,
test/Spec.hs) and against independent methods (dense diagonalisation of the
full 2^N Hamiltonian, brute-force orbit enumeration). CPU only."""
import itertools
import os

import numpy as np
import pytest

HEIS = np.array([[1, 0, 0, 0], [0, -1, 2, 0], [0, 2, -1, 0], [0, 0, 0, 1]], dtype=complex)
# the reference's source tree, when mounted (only for checks that read it)
REF = os.environ.get("SPINED_REFERENCE_DIR", "")


def ring(n, dist=1):
    return np.array([[i, (i + dist) % n] for i in range(n)])


def test_readme_ring4(oracle, pins):
    # README.md:37-50 config; README.md:62 dimension, README.md:91 energy.
    b = oracle.Basis(4, None, None, [])
    reps = b.build()
    assert len(reps) == pins["readme_ring4_dimension"]["value"]
    assert list(reps) == list(range(16))
    op = oracle.Operator(b, [oracle.Term(HEIS, np.array(pins["readme_ring4_sites"]["value"]))])
    e0 = np.linalg.eigvalsh(op.dense())[0]
    assert e0 == pytest.approx(pins["readme_ring4_e0"]["value"], abs=1e-12)


def test_spec_symmetry_pins(oracle, pins):
    p = pins["spec_periodicity"]["value"]
    assert oracle.symmetry_info(p["permutation"], p["sector"]) == p["periodicity"]
    for key in ("spec_invalid_permutation", "spec_invalid_sector"):
        v = pins[key]["value"]
        with pytest.raises(oracle.OracleError):
            oracle.symmetry_info(v["permutation"], v["sector"])


def test_spec_group_pins(oracle, pins):
    v = pins["spec_group_size"]["value"]
    g = oracle.group_closure(4, [(p, s) for p, s in v["generators"]])
    assert g.size == v["size_permutations"]
    b = oracle.Basis(4, None, 1, [(p, s) for p, s in v["generators"]])
    assert b.group_order == v["size_with_inversion"]
    bad = pins["spec_incompatible_sectors"]["value"]
    with pytest.raises(oracle.OracleError) as e:
        oracle.group_closure(4, [(p, s) for p, s in bad["generators"]])
    assert e.value.code == oracle.OR_INCOMPATIBLE_SYMMETRIES


def test_philox_known_answers(oracle):
    # Random123 known-answer vectors for philox4x32-10.
    assert oracle.philox4x32_10([0, 0, 0, 0], [0, 0]) == (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)
    assert oracle.philox4x32_10([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2) == (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)
    assert oracle.philox4x32_10([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0]) == (
        0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)
    v = oracle.start_vector(1234, 1001)
    assert v.min() >= -1.0 and v.max() < 1.0 and abs(v.mean()) < 0.1


def brute_orbit_min(x, perms, n, inv):
    imgs = []
    for p in perms:
        y = sum(((x >> p[i]) & 1) << i for i in range(n))
        imgs.append(y)
        if inv:
            imgs.append(~y & ((1 << n) - 1))
    return min(imgs)


@pytest.mark.parametrize("n,inv", [(8, None), (8, 1), (10, -1)])
def test_representatives_brute_force(oracle, n, inv):
    gens = [([(i + 1) % n for i in range(n)], 0), ([n - 1 - i for i in range(n)], 0)]
    b = oracle.Basis(n, n // 2, inv, gens)
    reps = b.build()
    g = oracle.group_closure(n, gens)
    expect = set()
    for bits in itertools.combinations(range(n), n // 2):
        x = sum(1 << k for k in bits)
        m = brute_orbit_min(x, g.perms, n, inv)
        if m == x and oracle.Basis.representative_weight(b, x):
            expect.add(x)
    assert list(reps) == sorted(expect)
    assert np.all(np.diff(reps.astype(np.int64)) > 0)


def full_space_hamiltonian(n, terms):
    H = np.zeros((2**n, 2**n), dtype=complex)
    for mat, sites in terms:
        k = sites.shape[1]
        for tup in sites:
            for x in range(2**n):
                a = 0
                for s in tup:
                    a = (a << 1) | ((x >> int(s)) & 1)
                for a2 in range(2**k):
                    v = mat[a2, a]
                    if v == 0:
                        continue
                    y = x
                    for m, s in enumerate(tup):
                        bit = (a2 >> (k - 1 - m)) & 1
                        y = (y & ~(1 << int(s))) | (bit << int(s))
                    H[y, x] += v
    return H


@pytest.mark.parametrize("n,j2", [(8, 0.0), (10, 0.3)])
def test_sector_spectra_match_full_space(oracle, n, j2):
    """Union of all (k, parity, inversion) sector spectra == full 2^n spectrum."""
    terms = [(HEIS, ring(n)), (j2 * HEIS, ring(n, 2))] if j2 else [(HEIS, ring(n))]
    full = np.linalg.eigvalsh(full_space_hamiltonian(n, terms))
    got = []
    for w in range(n + 1):
        for k in range(n):
            invs = [1, -1] if 2 * w == n else [None]
            for inv in invs:
                b = oracle.Basis(n, w, inv, [([(i + 1) % n for i in range(n)], k)])
                b.build()
                if len(b.reps) == 0:
                    continue
                op = oracle.Operator(b, [oracle.Term(m, s) for m, s in terms])
                H = op.dense()
                assert np.allclose(H, H.conj().T, atol=1e-12)
                got.extend(np.linalg.eigvalsh(H))
    assert len(got) == 2**n
    assert np.allclose(np.sort(got), full, atol=1e-10)


def test_chain24_sector_dimension(oracle):
    n = 24
    b = oracle.Basis(n, 12, 1, [([(i + 1) % n for i in range(n)], 0), ([n - 1 - i for i in range(n)], 0)])
    assert len(b.build()) == 28968


def test_square4x4_sector_dimension(oracle):
    from spined import lattices
    gens = lattices.square_symmetries(4)
    b = oracle.Basis(16, 8, 1, [(g, 0) for g in gens])
    assert b.group_order == 256
    assert len(b.build()) == 107


def test_lanczos_oracle_vs_eigsh(oracle):
    import scipy.sparse.linalg as sla
    n = 16
    b = oracle.Basis(n, 8, 1, [([(i + 1) % n for i in range(n)], 0), ([n - 1 - i for i in range(n)], 0)])
    b.build()
    op = oracle.Operator(b, [oracle.Term(HEIS, ring(n))])
    A = op.sparse()
    ev, psi, res, it = oracle.lanczos_ground_state(lambda v: A @ v, oracle.start_vector(1234, A.shape[0]))
    assert ev[0] == pytest.approx(sla.eigsh(A, k=1, which="SA")[0][0], rel=1e-12)
    assert res[0] <= 1e-8


def test_lattice_tables_match_reference_examples(pins):
    """The generated 6x6 / chain-40 tables equal the reference's example YAML
    (example/heisenberg_square_6x6.yaml, example/heisenberg_chain_40.yaml),
    as recorded in the golden pins."""
    from spined import lattices
    sq = pins["example_square6_tables"]["value"]
    assert sq["permutations"] == lattices.square_symmetries(6)
    assert sq["bonds"] == lattices.square_bonds(6)
    ch = pins["example_chain40_tables"]["value"]
    assert ch["translation"] == lattices.chain_translation(40)
    assert ch["parity"] == lattices.chain_parity(40)


@pytest.mark.skipif(not os.path.isdir(REF), reason="SPINED_REFERENCE_DIR does not name the reference tree")
def test_pins_regenerate_from_reference(pins, tmp_path):
    """The committed pins are what make_pins.py extracts from the reference."""
    import json
    import subprocess
    import sys
    here = os.path.dirname(os.path.abspath(__file__))
    pins_file = os.path.join(here, "golden", "reference_pins.json")
    before = open(pins_file).read()
    try:
        subprocess.check_call([sys.executable, os.path.join(here, "golden", "make_pins.py"), REF],
                              stdout=subprocess.DEVNULL)
        after = json.load(open(pins_file))
        assert {p["id"]: p for p in after["pins"]} == pins
    finally:
        with open(pins_file, "w") as f:
            f.write(before)


@pytest.mark.parametrize("n,w,inv,k", [(12, 6, 1, 0), (12, 6, -1, 6), (14, 5, None, 3), (10, None, 1, 0), (16, 8, -1, 0)])
def test_burnside_dimension_matches_enumeration(oracle, n, w, inv, k):
    from _burnside import sector_dimension
    gens = [([(i + 1) % n for i in range(n)], k)]
    if k in (0, n // 2):
        gens.append(([n - 1 - i for i in range(n)], 0))
    b = oracle.Basis(n, w, inv, gens)
    assert len(b.build()) == sector_dimension(b.group, n, w, inv)


def test_burnside_square4(oracle):
    from _burnside import sector_dimension
    from spined import lattices
    gens = [(g, 0) for g in lattices.square_symmetries(4)]
    b = oracle.Basis(16, 8, 1, gens)
    assert sector_dimension(b.group, 16, 8, 1) == 107 == len(b.build())


@pytest.mark.parametrize("n", [4, 6, 8, 10, 12, 14])
def test_bethe_ansatz_matches_dense(oracle, pins, n):
    """The Bethe-ansatz ring energy (tests/_bethe.py, an exact method that
    pins the chain workloads on the GPU) equals the oracle's sector matrix
    ground state; n = 4 is the README's -8."""
    from _bethe import heisenberg_ring_e0
    b = oracle.Basis(n, n // 2, None, [])
    op = oracle.Operator(b, [oracle.Term(HEIS, ring(n))])
    e0 = np.linalg.eigvalsh(op.dense().real)[0]
    assert heisenberg_ring_e0(n) == pytest.approx(e0, rel=1e-13, abs=1e-13)
    if n == 4:
        assert heisenberg_ring_e0(4) == pytest.approx(pins["readme_ring4_e0"]["value"], abs=1e-13)
