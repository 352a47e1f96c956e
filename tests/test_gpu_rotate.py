"""sed_rotate_vectors: the thick restart's basis rotation V[:, :kk] <- V Y
(D x m by m x kk, in place) on the tensor cores, by an error-free split of
the FP64 operands into 8-bit slices (exact in BF16) with exact FP32 sums in
tensor memory and integer recombination, against an FP64 product in numpy.

Tolerance: each operand is truncated to 56 bits below its row (V) or column
(Y) maximum, so an entry differs from the exact product by at most about
m 2^-55 max|V_r.| max|Y_.j| plus its own rounding; the test allows
1e-14 of m max|V_r.| max|Y_.j| (the FP64 reference carries errors of the same
order). The thick-restart solver gives the same eigenvalues with either
rotation path."""
import ctypes as C

import numpy as np
import pytest

from spined import lattices
from spined import _lib as L
from spined.model import build_model

pytestmark = pytest.mark.gpu


def _rotate(lib, V, Y, kk, path):
    import torch
    D, m = V.shape[0], V.shape[1]
    ld = D + 3
    Vd = torch.zeros((m, ld), dtype=torch.float64, device="cuda")
    Vd[:, :D] = torch.tensor(V.T)
    Yd = torch.tensor(np.ascontiguousarray(Y), dtype=torch.float64, device="cuda")
    st = lib.sed_rotate_vectors(C.c_void_p(Vd.data_ptr()), ld, m, C.c_void_p(Yd.data_ptr()), kk, D, path,
                                C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == 0, L.error_message(st)
    out = Vd[:, :D].cpu().numpy().T
    assert np.all(Vd[:, D:].cpu().numpy() == 0.0)  # nothing written beyond row D
    return out


@pytest.mark.parametrize("D,m,kk", [(1, 1, 1), (127, 4, 2), (1000, 12, 6), (4099, 16, 16), (3001, 17, 8),
                                    (20000, 32, 16), (129, 32, 1)])
def test_tensor_rotation_matches_fp64(sed, D, m, kk):
    lib = L.load()
    rng = np.random.default_rng(D + 31 * m + kk)
    V = rng.normal(size=(D, m)) * np.exp(rng.uniform(-3, 3, size=(D, 1)))  # rows of different scales
    V[rng.random(size=(D, m)) < 0.05] = 0.0
    if D > 10:
        V[3] = 0.0                      # a zero row
        V[5] *= 1e-200                  # tiny and huge rows
        V[7] *= 1e200
        V[9, 0] = 5e-310                # a subnormal entry
    Y = rng.normal(size=(m, kk)) * np.exp(rng.uniform(-2, 2, size=(1, kk)))
    want = V @ Y
    got = _rotate(lib, V, Y, kk, L.SED_ROTATE_TENSOR)
    scale = m * np.abs(V).max(axis=1, keepdims=True) * np.abs(Y).max(axis=0, keepdims=True)
    assert np.all(np.abs(got[:, :kk] - want) <= 1e-14 * scale + 1e-300)
    np.testing.assert_array_equal(got[:, kk:], V[:, kk:])  # untouched columns
    fp = _rotate(lib, V, Y, kk, L.SED_ROTATE_FP64)
    assert np.all(np.abs(fp[:, :kk] - want) <= 1e-14 * scale + 1e-300)


def test_tensor_rotation_nan_and_errors(sed):
    lib = L.load()
    rng = np.random.default_rng(5)
    V = rng.normal(size=(300, 8))
    V[17, 3] = np.nan
    Y = rng.normal(size=(8, 4))
    got = _rotate(lib, V, Y, 4, L.SED_ROTATE_TENSOR)
    assert np.all(np.isnan(got[17, :4]))
    assert np.all(np.isfinite(np.delete(got, 17, axis=0)))
    import torch
    Vd = torch.zeros((20, 64), dtype=torch.float64, device="cuda")
    Yd = torch.zeros((20, 17), dtype=torch.float64, device="cuda")
    st = lib.sed_rotate_vectors(C.c_void_p(Vd.data_ptr()), 64, 20, C.c_void_p(Yd.data_ptr()), 17, 64,
                                L.SED_ROTATE_TENSOR, None)
    assert st == L.LS_INVALID_ARGUMENT  # kk > 16 is not a tensor-core shape
    st = lib.sed_rotate_vectors(C.c_void_p(Vd.data_ptr()), 64, 20, C.c_void_p(Yd.data_ptr()), 17, 64,
                                L.SED_ROTATE_AUTO, None)
    assert st == 0  # AUTO takes the FP64 kernel for kk > 16


def test_thick_restart_rotation_paths_agree(sed, oracle):
    lib = L.load()
    m = lattices.heisenberg_chain(22, j2=0.3)
    built = build_model(m)
    res = {}
    try:
        for path in (L.SED_ROTATE_FP64, L.SED_ROTATE_TENSOR):
            lib.sed_set_rotate_path(path)
            res[path] = sed.eigh(built.hamiltonian, nev=2, tol=1e-9, max_basis=12)
    finally:
        lib.sed_set_rotate_path(L.SED_ROTATE_AUTO)
    a, b = res[L.SED_ROTATE_FP64], res[L.SED_ROTATE_TENSOR]
    assert a.restarts >= 1 and b.restarts >= 1  # the rotation ran
    np.testing.assert_allclose(b.eigenvalues, a.eigenvalues, rtol=1e-12)
    assert np.all(b.residuals <= 1e-9)
