"""ls_build on the GPU: representatives and stabiliser norms bit-exact
against the oracle (src/SpinED/Internal.hs:178-182,230-254)."""
import numpy as np
import pytest

from _models import both
from spined import lattices

pytestmark = pytest.mark.gpu

CASES = {
    "readme_ring4": lattices.Model("ring4", 4, None, None, [], [(lattices.HEISENBERG, lattices.chain_bonds(4))]),
    "chain24": lattices.heisenberg_chain(24),
    "chain16_k3": lattices.heisenberg_chain(16, momentum=3, parity=None),
    "chain18_k9_odd": lattices.heisenberg_chain(18, momentum=9, parity=1, spin_inversion=-1),
    "chain14_w5": lattices.heisenberg_chain(14, hamming_weight=5, spin_inversion=None),
    "square4": lattices.heisenberg_square(4),
    "square4_inv-": lattices.heisenberg_square(4, spin_inversion=-1),
    "ring10_nohw_inv": lattices.Model("r10", 10, None, 1, [(lattices.chain_translation(10), 0)],
                                      [(lattices.HEISENBERG, lattices.chain_bonds(10))]),
    "chain34_k0": lattices.heisenberg_chain(34),  # 64-bit words, D ~ 1.7e6? (large)
    # tori: the top-row pruning of the scan with momentum (pi, pi), without a
    # Hamming weight, and on a 6x4 torus (rows of 6 sites, 4 rows)
    "square4_kpi": lattices.Model("sq4kpi", 16, 8, 1, [(g, 2) for g in lattices.square_symmetries(4)[:2]],
                                  [(lattices.HEISENBERG, lattices.square_bonds(4))]),
    "square4_nohw": lattices.Model("sq4nohw", 16, None, 1, [(g, 0) for g in lattices.square_symmetries(4)],
                                   [(lattices.HEISENBERG, lattices.square_bonds(4))]),
    "torus6x4_w11": lattices.Model("t6x4", 24, 11, None, [(g, 0) for g in lattices.rect_translations(6, 4)],
                                   [(lattices.HEISENBERG, lattices.rect_bonds(6, 4))]),
    # line tables: rotations without reflections (rows and columns in one
    # direction each), and reflections of a 6x4 torus (rows only)
    "square4_C4": lattices.Model("sq4c4", 16, 8, 1,
                                 [(g, 0) for g in lattices.square_symmetries(4)[:2] + lattices.square_symmetries(4)[4:]],
                                 [(lattices.HEISENBERG, lattices.square_bonds(4))]),
    "torus6x4_refl": lattices.Model("t6x4r", 24, 12, 1, [(g, 0) for g in lattices.rect_translations(6, 4)] + [
        ([(y * 6) + (5 - x) for y in range(4) for x in range(6)], 0),
        ([((3 - y) * 6) + x for y in range(4) for x in range(6)], 0)],
        [(lattices.HEISENBERG, lattices.rect_bonds(6, 4))]),
}


@pytest.mark.parametrize("name", [k for k in CASES if k != "chain34_k0"])
def test_representatives_bit_exact(sed, oracle, name):
    built, ob, _ = both(sed, oracle, CASES[name])
    reps = sed.basis_get_states(built.basis)
    assert reps.dtype == np.uint64
    assert np.array_equal(reps, ob.reps)
    assert sed.get_number_states(built.basis) == len(ob.reps)
    norms = built.basis.norms()
    assert np.array_equal(norms, ob.norms())  # sqrt(S/|G|), same IEEE ops


def test_readme_dimension(sed, pins):
    built, _, _ = both(sed, __import__("oracle"), CASES["readme_ring4"])
    reps = sed.basis_get_states(built.basis)
    assert len(reps) == pins["readme_ring4_dimension"]["value"]
    assert list(reps) == list(range(16))


def test_build_unsafe_round_trip(sed, oracle):
    m = lattices.heisenberg_chain(20)
    built, ob, _ = both(sed, oracle, m)
    reps = sed.basis_get_states(built.basis)
    from spined.model import build_model
    fresh = build_model(m, build=False)
    sed.build_basis(fresh.basis, reps)  # the resume path, src/SpinED.hs:319-331
    assert np.array_equal(sed.basis_get_states(fresh.basis), reps)
    assert np.array_equal(fresh.basis.norms(), built.basis.norms())
    bad = reps.copy()
    bad[3] = bad[3] + 1  # not a representative (or unsorted)
    with pytest.raises(sed.LatticeSymmetriesException):
        sed.build_basis(build_model(m, build=False).basis, bad)
    with pytest.raises(sed.LatticeSymmetriesException):
        sed.build_basis(build_model(m, build=False).basis, reps[::-1].copy())


def test_index_lookup(sed, oracle):
    built, ob, _ = both(sed, oracle, lattices.heisenberg_square(4))
    for i, r in enumerate(ob.reps):
        assert built.basis.index(int(r)) == i
    assert built.basis.index(int(ob.reps[-1]) + 1) is None


def test_large_chain_properties(sed, oracle):
    """34 spins (64-bit words): count from the oracle on a slice, sortedness,
    and every sampled output is an orbit minimum with a nonzero norm."""
    m = CASES["chain34_k0"]
    from spined.model import build_model
    built = build_model(m)
    reps = sed.basis_get_states(built.basis)
    assert np.all(np.diff(reps.astype(np.int64)) > 0)
    ob = oracle.Basis(m.number_spins, m.hamming_weight, m.spin_inversion, m.symmetries)
    rng = np.random.default_rng(1)
    for r in rng.choice(reps, 2000, replace=False):
        assert ob.representative_weight(int(r)) > 0
    # the first 2^22 ranks of the word space, counted by the oracle
    part = ob.build(0, 1 << 22)
    assert np.array_equal(reps[: len(part)], part)
