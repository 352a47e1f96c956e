"""sed_eigh_batched: many J1-J2 chains of uneven size in one persistent
launch (block Lanczos, block size 4; FP64 vectors and matvec, double-float
Gram-Schmidt products), against the FP64 oracle.

Small batches are compared eigenvalue by eigenvalue with dense
diagonalisations of the oracle's sector matrices (1e-10 relative) and every
returned eigenpair's residual ||H psi - E psi|| <= 1e-8 is recomputed by the
oracle. The 128-chain workload (N uniform over 16..28, J2/J1 uniform in
[0, 0.6], seed 2024) is checked through size-independent properties:
residuals recomputed through ls_operator_matmat, orthonormal eigenvectors,
ascending eigenvalues, and agreement with the single-operator solver on
its largest chains."""
import numpy as np
import pytest

from _models import both
from spined import lattices
from spined.model import build_model

pytestmark = pytest.mark.gpu

EV_RTOL = 1e-10
RES_TOL = 1e-8


def _check_pairs(oop, evals, vecs):
    for k, E in enumerate(evals):
        psi = vecs[:, k]
        assert abs(np.linalg.norm(psi) - 1.0) < 1e-10
        hp = oop.matvec(psi.astype(np.complex128)).real
        assert np.linalg.norm(hp - E * psi) <= RES_TOL * 1.01


@pytest.mark.parametrize("nev", [4, 2])
def test_small_batch_matches_oracle(sed, oracle, nev):
    rng = np.random.default_rng(7 + nev)
    models = [lattices.heisenberg_chain(int(n), j2=float(j))
              for n, j in zip(rng.choice([10, 12, 14, 16, 18], size=9), rng.uniform(0, 0.6, size=9))]
    pairs = [both(sed, oracle, m) for m in models]
    res = sed.eigh_batched([b.hamiltonian for b, _, _ in pairs], nev=nev)
    for i, (b, ob, oop) in enumerate(pairs):
        want = np.linalg.eigvalsh(oop.dense().real)[:nev]
        np.testing.assert_allclose(res.eigenvalues[i], want, rtol=EV_RTOL, atol=0)
        assert np.all(res.residuals[i] <= RES_TOL)
        _check_pairs(oop, res.eigenvalues[i], res.eigenvectors[i])


def test_one_problem_and_more_problems_than_ctas_agree(sed, oracle):
    """The same operator solved alone and inside a batch of 400 (more
    problems than CTAs: groups then queue several problems each)."""
    m = lattices.heisenberg_chain(14, j2=0.3)
    b0, ob, oop = both(sed, oracle, m)
    alone = sed.eigh_batched([b0.hamiltonian], nev=4)
    many = [build_model(lattices.heisenberg_chain(12 + 2 * (i % 3), j2=0.1 * (i % 6))) for i in range(399)]
    res = sed.eigh_batched([b0.hamiltonian] + [x.hamiltonian for x in many], nev=4, vectors=False)
    want = np.linalg.eigvalsh(oop.dense().real)[:4]
    np.testing.assert_allclose(alone.eigenvalues[0], want, rtol=EV_RTOL)
    np.testing.assert_allclose(res.eigenvalues[0], want, rtol=EV_RTOL)
    assert np.all(res.residuals <= RES_TOL)


def test_batched_rejects_bad_arguments(sed):
    b = build_model(lattices.heisenberg_chain(12))
    with pytest.raises(sed.LatticeSymmetriesException):
        sed.eigh_batched([b.hamiltonian], nev=5)
    with pytest.raises(sed.LatticeSymmetriesException):
        c = build_model(lattices.heisenberg_chain(16, momentum=3, parity=None))  # complex characters
        sed.eigh_batched([c.hamiltonian], nev=2)


def test_j1j2_chains_128(sed):
    import ctypes as C
    from spined import _lib as L
    models = lattices.j1j2_chains(128, seed=2024)
    built = [build_model(m) for m in models]
    res = sed.eigh_batched([b.hamiltonian for b in built], nev=4)
    assert res.eigenvalues.shape == (128, 4)
    assert np.all(res.residuals <= RES_TOL)
    assert np.all(np.diff(res.eigenvalues, axis=1) >= -1e-12)
    lib = L.load()
    for i in range(0, 128, 9):  # independent residual check through the C ABI
        v = res.eigenvectors[i]
        D = v.shape[0]
        np.testing.assert_allclose(v.T @ v, np.eye(4), atol=1e-10)
        hv = np.zeros_like(v, order="F")
        sed.check_status(lib.ls_operator_matmat(built[i].hamiltonian.ptr, 1, D, 4, C.c_void_p(v.ctypes.data), D,
                                                C.c_void_p(hv.ctypes.data), D))
        r = np.linalg.norm(hv - v * res.eigenvalues[i][None, :], axis=0)
        assert np.all(r <= RES_TOL * 1.01), (i, r)
    # the largest chains against the single-operator Lanczos (nev = 4)
    big = sorted(range(128), key=lambda i: -models[i].number_spins)[:2]
    for i in big:
        one = sed.eigh(built[i].hamiltonian, nev=4)
        np.testing.assert_allclose(res.eigenvalues[i], one.eigenvalues, rtol=EV_RTOL)


@pytest.mark.parametrize("threads,per_sm", [(128, 1), (128, 2), (256, 1), (256, 2)])
def test_fixed_launch_shapes_agree(sed, oracle, threads, per_sm):
    """Every launch shape the autotuner chooses among gives the same pairs:
    each shape, fixed through sed_set_batched_launch, against dense
    diagonalisation of the oracle's sector matrices."""
    from spined import _lib as L
    lib = L.load()
    models = [lattices.heisenberg_chain(n, j2=0.1 * k) for k, n in enumerate((12, 14, 16, 18, 14))]
    pairs = [both(sed, oracle, m) for m in models]
    try:
        lib.sed_set_batched_launch(threads, per_sm)
        res = sed.eigh_batched([b.hamiltonian for b, _, _ in pairs], nev=4)
    finally:
        lib.sed_set_batched_launch(0, 0)
    assert res.ctas_per_sm == per_sm
    for i, (b, ob, oop) in enumerate(pairs):
        want = np.linalg.eigvalsh(oop.dense().real)[:4]
        np.testing.assert_allclose(res.eigenvalues[i], want, rtol=EV_RTOL, atol=0)
        assert np.all(res.residuals[i] <= RES_TOL)
