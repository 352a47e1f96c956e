"""Parity at the workloads' full sizes, where the GPU paths differ from the
small cases: the 6x6 lattice (D = 15 804 956; the scan's top-row pruning and
line tables, the orbit-table recording of the stream form), the 36- and
40-site chains (64-bit words) and the 128-chain batch.

- Representatives and norms are compared bit for bit with the oracle's own
  enumeration (src/SpinED/Internal.hs:178-182,238-254) on word-rank slices
  spread over the sector.
- Rows of H x (src/SpinED/Internal.hs:411-429) are compared with the
  oracle's pull-form rows, index lookups included, at 1e-12 of max|y|.
- Ground-state energies are pinned by independent exact results: the Bethe
  ansatz for the rings (1e-10 relative) and the published 6x6 value
  E0/N = -0.678872 J per site for sum S.S (Schulz, Ziman & Poilblanc,
  J. Phys. I France 6, 675 (1996)); the 6x6 eigenpair is also checked row
  by row against the oracle's H.
- For the 128-chain batch, sampled chains' 4 returned eigenvalues are the
  lowest 4 of the oracle's sector matrix (scipy eigsh).
"""
from math import comb

import numpy as np
import pytest

from _bethe import heisenberg_ring_e0
from spined import lattices
from spined import _lib as L

pytestmark = pytest.mark.gpu

RTOL_MV = 1e-12   # FP64 rows: summation order only
EV_RTOL = 1e-10   # eigenvalues against exact values


def colex_rank(word: int, n: int) -> int:
    r, i = 0, 0
    for p in range(n):
        if (word >> p) & 1:
            i += 1
            r += comb(p, i)
    return r


def colex_unrank(r: int, n: int, w: int) -> int:
    word = 0
    for i in range(w, 0, -1):
        p = i - 1
        while p + 1 < n and comb(p + 1, i) <= r:
            p += 1
        word |= 1 << p
        r -= comb(p, i)
    return word


def _slices_around(reps: np.ndarray, n: int, w: int, count: int, width: int, rng) -> list[tuple[int, int]]:
    """`count` rank slices of `width` words centred on representatives at
    evenly spaced quantiles of the list (where the scan finds survivors),
    plus two slices at random ranks of the whole word space."""
    space = comb(n, w)
    out = []
    for q in np.linspace(0.0, 1.0, count):
        r = colex_rank(int(reps[min(len(reps) - 1, int(q * (len(reps) - 1)))]), n)
        lo = max(0, r - width // 2)
        out.append((lo, min(space, lo + width)))
    for r in rng.integers(0, space - width, size=2):
        out.append((int(r), int(r) + width))
    return out


def _check_slices(reps, norms, ob, n, w, slices):
    G = ob.group_order
    for lo, hi in slices:
        want, wts = ob.slice(lo, hi)
        a = np.searchsorted(reps, np.uint64(colex_unrank(lo, n, w)))
        b = np.searchsorted(reps, np.uint64(colex_unrank(hi, n, w))) if hi < comb(n, w) else len(reps)
        assert np.array_equal(reps[a:b], want), (lo, hi)
        assert np.array_equal(norms[a:b], np.sqrt(wts.astype(np.float64) / float(G))), (lo, hi)


@pytest.fixture(scope="module")
def square6(sed, oracle):
    from spined.model import build_model
    m = lattices.heisenberg_square(6)
    built = build_model(m)
    reps = sed.basis_get_states(built.basis).copy()
    norms = built.basis.norms()
    ob = oracle.Basis(m.number_spins, m.hamming_weight, m.spin_inversion, m.symmetries)
    oop = oracle.Operator(ob, [oracle.Term(np.array(a, dtype=complex), np.array(s)) for a, s in m.terms],
                          build=False)
    return m, built, reps, norms, ob, oop


def _weights(norms, G):
    return np.rint(norms * norms * G).astype(np.uint32)


def test_square6_representatives_on_rank_slices(square6):
    m, built, reps, norms, ob, _ = square6
    assert len(reps) == 15_804_956
    assert np.all(np.diff(reps.astype(np.int64)) > 0)
    _check_slices(reps, norms, ob, 36, 18, _slices_around(reps, 36, 18, 8, 1 << 21, np.random.default_rng(1)))


def test_square6_matrix_rows_match_oracle(sed, square6):
    """Rows of H x through the orbit-table stream form and the on-the-fly
    form, against the oracle's rows over the same representative list."""
    import torch
    m, built, reps, norms, ob, oop = square6
    op = built.hamiltonian
    op.prepare(L.SED_FORM_STREAM)
    D = len(reps)
    lib = L.load()
    assert lib.sed_operator_recorded_with_table(op.ptr) == 1
    g = torch.Generator(device="cuda").manual_seed(12)
    x = torch.randn(D, dtype=torch.float64, device="cuda", generator=g)
    y = sed.apply(op, x)
    from spined.model import build_model
    otf = build_model(m, build=False)
    sed.build_basis(otf.basis, reps)
    otf.hamiltonian.prepare(L.SED_FORM_ON_THE_FLY)
    y_otf = sed.apply(otf.hamiltonian, x)
    torch.cuda.synchronize()
    assert torch.equal(y, y_otf)  # same sum in the same order
    xh, yh = x.cpu().numpy().astype(np.complex128), y.cpu().numpy()
    w = _weights(norms, ob.group_order)
    scale = np.abs(yh).max()
    rng = np.random.default_rng(5)
    starts = np.concatenate([[0, D - 2000], rng.integers(0, D - 2000, size=10)])
    for a in starts:
        want = oop.matvec_rows(reps, w, xh, int(a), int(a) + 2000).real
        np.testing.assert_allclose(yh[a:a + 2000], want, rtol=0, atol=RTOL_MV * scale)


def test_square6_ground_state(sed, square6):
    """E0 against the published 6x6 value, and the eigenpair against the
    oracle's H on sampled rows: |(H psi)_i - E psi_i| <= the residual bound."""
    import torch
    m, built, reps, norms, ob, oop = square6
    D = len(reps)
    out = torch.empty(D, dtype=torch.float64, device="cuda")
    r = sed.eigh(built.hamiltonian, tol=1e-8, seed=1234, out=out)
    E = float(r.eigenvalues[0])
    assert r.residuals[0] <= 1e-8
    assert abs(E / (4 * 36) - (-0.678872)) <= 1e-6  # published to 6 digits
    psi = out.cpu().numpy()
    assert abs(np.linalg.norm(psi) - 1.0) < 1e-12
    psi_c = psi.astype(np.complex128)
    w = _weights(norms, ob.group_order)
    rng = np.random.default_rng(6)
    for a in rng.integers(0, D - 2000, size=6):
        hp = oop.matvec_rows(reps, w, psi_c, int(a), int(a) + 2000).real
        assert np.max(np.abs(hp - E * psi[a:a + 2000])) <= 1e-8
    # the FP32-stored form reaches the same eigenvalue
    r2 = sed.eigh(built.hamiltonian, tol=1e-8, seed=1234, out=out, precision=L.SED_PRECISION_MIXED)
    assert r2.residuals[0] <= 1e-8
    assert abs(r2.eigenvalues[0] - E) <= EV_RTOL * abs(E)


def test_chain24_ground_state_bethe(sed):
    """The chain-24 workload (k = 0, P = +1, Z = +1) holds the ring's
    ground state: its eigenvalue equals the Bethe-ansatz energy."""
    from spined.model import build_model
    built = build_model(lattices.heisenberg_chain(24))
    assert sed.get_number_states(built.basis) == 28_968
    r = sed.eigh(built.hamiltonian, tol=1e-8, seed=1234)
    e = heisenberg_ring_e0(24)
    assert abs(r.eigenvalues[0] - e) <= EV_RTOL * abs(e)
    assert r.residuals[0] <= 1e-8


def test_chain36_representatives_and_rows(sed, oracle):
    """64-bit words on a large chain (D ~ 6.3e7): rank slices bit-exact and
    sampled rows of H x against the oracle."""
    import torch
    from spined.model import build_model
    m = lattices.heisenberg_chain(36)
    built = build_model(m)
    reps = sed.basis_get_states(built.basis).copy()
    norms = built.basis.norms()
    ob = oracle.Basis(36, 18, 1, m.symmetries)
    _check_slices(reps, norms, ob, 36, 18, _slices_around(reps, 36, 18, 8, 1 << 21, np.random.default_rng(2)))
    op = built.hamiltonian
    op.prepare(L.SED_FORM_STREAM)
    D = len(reps)
    g = torch.Generator(device="cuda").manual_seed(13)
    x = torch.randn(D, dtype=torch.float64, device="cuda", generator=g)
    y = sed.apply(op, x)
    torch.cuda.synchronize()
    xh, yh = x.cpu().numpy().astype(np.complex128), y.cpu().numpy()
    del x, y
    oop = oracle.Operator(ob, [oracle.Term(np.array(a, dtype=complex), np.array(s)) for a, s in m.terms],
                          build=False)
    w = _weights(norms, ob.group_order)
    scale = np.abs(yh).max()
    for a in np.concatenate([[0, D - 2000], np.random.default_rng(7).integers(0, D - 2000, size=6)]):
        want = oop.matvec_rows(reps, w, xh, int(a), int(a) + 2000).real
        np.testing.assert_allclose(yh[a:a + 2000], want, rtol=0, atol=RTOL_MV * scale)


def test_chain40_representatives_and_ground_state(sed, oracle):
    """The chain-40 workload (D = 861 725 794, 6.9 GB of representatives):
    the count equals Burnside's, rank slices are bit-exact against the
    oracle, and the thick-restart solver in FP64 and in the FP32-stored form
    both reach the Bethe-ansatz energy."""
    import torch
    from _burnside import sector_dimension
    from spined.model import build_model
    torch.cuda.empty_cache()
    L.load().sed_release_workspace()  # earlier tests' cached Krylov vectors
    m = lattices.heisenberg_chain(40)
    built = build_model(m)
    D = sed.get_number_states(built.basis)
    ob = oracle.Basis(40, 20, 1, m.symmetries)
    assert D == sector_dimension(ob.group, 40, 20, 1) == 861_725_794
    # the sorted list stays on the device; slices are located there
    ptr = L.load().sed_basis_device_states(built.basis.ptr)

    class _Dev:
        __cuda_array_interface__ = {"shape": (D,), "typestr": "<i8", "data": (ptr, False), "version": 2}

    dev = torch.as_tensor(_Dev(), device="cuda")  # 40-bit words: int64 view of the uint64 list
    assert bool((dev[1:] > dev[:-1]).all())
    G = ob.group_order
    rng = np.random.default_rng(3)
    picks = [int(dev[(D - 1) * q // 7].item()) for q in range(8)]  # exact integer positions < D
    space = comb(40, 20)
    slices = [(max(0, colex_rank(v, 40) - (1 << 20)), max(0, colex_rank(v, 40) - (1 << 20)) + (1 << 21))
              for v in picks]
    slices += [(int(r), int(r) + (1 << 21)) for r in rng.integers(0, space - (1 << 21), size=2)]
    for lo, hi in slices:
        assert hi < space
        want, wts = ob.slice(lo, hi)
        bounds = torch.tensor([colex_unrank(lo, 40, 20), colex_unrank(hi, 40, 20)], dtype=torch.int64,
                              device="cuda")
        a, b = [int(v) for v in torch.searchsorted(dev, bounds).cpu()]
        got = dev[a:b].cpu().numpy().astype(np.uint64)
        assert np.array_equal(got, want), (lo, hi)
        for k in range(0, len(want), max(1, len(want) // 16)):  # the device index agrees
            assert built.basis.index(int(want[k])) == a + k
    del dev
    e = heisenberg_ring_e0(40)
    out = torch.empty(D, dtype=torch.float64, device="cuda")
    r64 = sed.eigh(built.hamiltonian, tol=1e-8, seed=1234, max_basis=12, out=out)
    assert r64.residuals[0] <= 1e-8
    assert abs(r64.eigenvalues[0] - e) <= EV_RTOL * abs(e)
    r32 = sed.eigh(built.hamiltonian, tol=1e-8, seed=1234, max_basis=16, out=out,
                   precision=L.SED_PRECISION_MIXED)
    assert r32.residuals[0] <= 1e-8
    assert abs(r32.eigenvalues[0] - e) <= EV_RTOL * abs(e)


def test_batch128_lowest_four_are_lowest(sed, oracle):
    """The 128-chain batch (seed 2024): on a sample of chains — the
    largest, the smallest and four at random — the 4 returned eigenvalues
    are the 4 lowest of the oracle's sector matrix (scipy eigsh)."""
    import scipy.sparse.linalg as sla
    from spined.model import build_model
    models = lattices.j1j2_chains(128, seed=2024)
    built = [build_model(mm) for mm in models]
    res = sed.eigh_batched([b.hamiltonian for b in built], nev=4, vectors=False)
    assert np.all(res.residuals <= 1e-8)
    dims = np.array([sed.get_number_states(b.basis) for b in built])
    rng = np.random.default_rng(4)
    sample = sorted({int(np.argmax(dims)), int(np.argmin(dims)), *rng.choice(128, 4, replace=False).tolist()})
    for i in sample:
        mm = models[i]
        ob = oracle.Basis(mm.number_spins, mm.hamming_weight, mm.spin_inversion, mm.symmetries)
        oop = oracle.Operator(ob, [oracle.Term(np.array(a, dtype=complex), np.array(s)) for a, s in mm.terms])
        A = oop.sparse()
        want = np.sort(sla.eigsh(A, k=6, which="SA", tol=1e-13)[0])[:4]
        np.testing.assert_allclose(res.eigenvalues[i], want, rtol=EV_RTOL, atol=1e-12, err_msg=f"chain {i}")
