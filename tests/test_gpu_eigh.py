"""sed_eigh (the device Lanczos replacing PRIMME at src/SpinED.hs:404)
against the FP64 oracle: eigenvalues within 1e-10 relative, residual
||H psi - E psi|| <= 1e-8 recomputed independently."""
import numpy as np
import pytest

from _models import both, random_complex_term
from spined import lattices

pytestmark = pytest.mark.gpu

EV_RTOL = 1e-10
RES_TOL = 1e-8


def check_pair(oop, E, psi, tol=RES_TOL):
    psi = psi / np.linalg.norm(psi)
    hp = oop.matvec(psi.astype(np.complex128))
    if oop.is_real:
        hp = hp.real
    r = np.linalg.norm(hp - E * psi)
    assert r <= tol * 1.01, r


def test_readme_ground_state(sed, oracle, pins):
    m = lattices.Model("ring4", 4, None, None, [], [(lattices.HEISENBERG, pins["readme_ring4_sites"]["value"])])
    built, ob, oop = both(sed, oracle, m)
    res = sed.eigh(built.hamiltonian)
    assert res.eigenvalues[0] == pytest.approx(pins["readme_ring4_e0"]["value"], abs=1e-10)
    assert res.residuals[0] <= RES_TOL
    check_pair(oop, res.eigenvalues[0], res.eigenvectors[:, 0])


@pytest.mark.parametrize("name,model", [
    ("chain24", lattices.heisenberg_chain(24)),
    ("chain20_j2", lattices.heisenberg_chain(20, j2=0.4)),
    ("square4", lattices.heisenberg_square(4)),
])
def test_ground_state_matches_oracle(sed, oracle, name, model):
    built, ob, oop = both(sed, oracle, model)
    A = oop.sparse()
    ev, _, _, _ = oracle.lanczos_ground_state(lambda v: A @ v, oracle.start_vector(1234, A.shape[0]))
    res = sed.eigh(built.hamiltonian, seed=1234)
    assert res.eigenvalues[0] == pytest.approx(ev[0], rel=EV_RTOL)
    assert res.residuals[0] <= RES_TOL
    check_pair(oop, res.eigenvalues[0], res.eigenvectors[:, 0])


def test_lowest_four(sed, oracle):
    import scipy.sparse.linalg as sla
    built, ob, oop = both(sed, oracle, lattices.heisenberg_chain(18, j2=0.3))
    A = oop.sparse()
    want = np.sort(sla.eigsh(A, k=4, which="SA")[0])
    res = sed.eigh(built.hamiltonian, nev=4)
    np.testing.assert_allclose(np.sort(res.eigenvalues), want, rtol=EV_RTOL)
    assert np.all(res.residuals <= RES_TOL)


def test_complex_sector(sed, oracle):
    import scipy.sparse.linalg as sla
    m = lattices.heisenberg_chain(16, momentum=3, parity=None, spin_inversion=None)
    built, ob, oop = both(sed, oracle, m)
    assert not oop.is_real
    A = oop.sparse()
    want = sla.eigsh(A, k=1, which="SA")[0][0]
    res = sed.eigh(built.hamiltonian, dtype=np.complex128)
    assert res.eigenvalues[0] == pytest.approx(want, rel=EV_RTOL)
    check_pair(oop, res.eigenvalues[0], res.eigenvectors[:, 0])


def test_float32_output(sed, oracle):
    built, ob, oop = both(sed, oracle, lattices.heisenberg_chain(20))
    res = sed.eigh(built.hamiltonian, dtype=np.float32)
    assert res.eigenvectors.dtype == np.float32
    A = oop.sparse()
    ev, _, _, _ = oracle.lanczos_ground_state(lambda v: A @ v, oracle.start_vector(1234, A.shape[0]))
    assert res.eigenvalues[0] == pytest.approx(ev[0], rel=EV_RTOL)


def test_start_vector_philox_parity(sed, oracle):
    """A run limited to the start vector's Rayleigh quotient: the device
    Philox stream equals the oracle's, so one step from the same seed sees
    the same alpha_0."""
    built, ob, oop = both(sed, oracle, lattices.heisenberg_chain(16))
    v = oracle.start_vector(77, len(ob.reps))
    res = sed.eigh(built.hamiltonian, seed=77)
    res2 = sed.eigh(built.hamiltonian, start=v / np.linalg.norm(v))
    assert res.eigenvalues[0] == pytest.approx(res2.eigenvalues[0], rel=1e-12)
    assert res.iterations == res2.iterations


@pytest.mark.parametrize("name,model", [
    ("chain24", lattices.heisenberg_chain(24)),
    ("chain20_j2", lattices.heisenberg_chain(20, j2=0.45)),
    ("square4_inv-", lattices.heisenberg_square(4, spin_inversion=-1)),
])
def test_mixed_precision_matches_fp64_oracle(sed, oracle, name, model):
    """FP32-stored Krylov cycles anchored on an FP64 vector: eigenvalue within
    1e-10 relative of the FP64 oracle, residual <= 1e-8 (recomputed here)."""
    from spined import _lib as L
    built, ob, oop = both(sed, oracle, model)
    A = oop.sparse()
    ev, _, _, _ = oracle.lanczos_ground_state(lambda v: A @ v, oracle.start_vector(1234, A.shape[0]))
    res = sed.eigh(built.hamiltonian, seed=1234, precision=L.SED_PRECISION_MIXED)
    assert res.fp32_iterations > 0
    assert res.eigenvalues[0] == pytest.approx(ev[0], rel=EV_RTOL)
    assert res.residuals[0] <= RES_TOL
    check_pair(oop, res.eigenvalues[0], res.eigenvectors[:, 0])


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("name,model,m", [
    ("chain24", lattices.heisenberg_chain(24), 16),
    ("chain20_j2", lattices.heisenberg_chain(20, j2=0.45), 8),
    ("square4", lattices.heisenberg_square(4), 6),
])
def test_thick_restart_matches_fp64_oracle(sed, oracle, name, model, m, precision):
    """Thick-restart Lanczos with at most m stored vectors (max_basis <= 32),
    FP64 or FP32-stored with an FP64 refinement: eigenvalue within 1e-10
    relative of the FP64 oracle, residual <= 1e-8 (recomputed here)."""
    from spined import _lib as L
    built, ob, oop = both(sed, oracle, model)
    A = oop.sparse()
    ev, _, _, _ = oracle.lanczos_ground_state(lambda v: A @ v, oracle.start_vector(1234, A.shape[0]))
    p = L.SED_PRECISION_FP64 if precision == "fp64" else L.SED_PRECISION_MIXED
    res = sed.eigh(built.hamiltonian, seed=1234, max_basis=m, precision=p)
    if precision == "mixed":
        assert res.fp32_iterations > 0
    if A.shape[0] > m:
        assert res.restarts > 0  # the basis really was recycled
    assert res.eigenvalues[0] == pytest.approx(ev[0], rel=EV_RTOL)
    assert res.residuals[0] <= RES_TOL
    check_pair(oop, res.eigenvalues[0], res.eigenvectors[:, 0])


def test_thick_restart_lowest_three(sed, oracle):
    import scipy.sparse.linalg as sla
    built, ob, oop = both(sed, oracle, lattices.heisenberg_chain(18, j2=0.3))
    want = np.sort(sla.eigsh(oop.sparse(), k=3, which="SA")[0])
    res = sed.eigh(built.hamiltonian, nev=3, max_basis=12)
    np.testing.assert_allclose(res.eigenvalues, want, rtol=EV_RTOL)
    assert np.all(res.residuals <= RES_TOL)
    for k in range(3):
        check_pair(oop, res.eigenvalues[k], res.eigenvectors[:, k])
