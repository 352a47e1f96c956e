"""sed_operator_expectation_noalloc: the expectation entry point for callers
that cannot let a library allocate device memory (their device memory belongs
to their own pool allocator, or cudaMalloc's implicit synchronisation is too
costly for them). Called through the C ABI and checked against the existing
ls_operator_expectation / ls_operator_matmat on two calls in a row.

This file is collected last on purpose; it passes alone in a fresh process
and after the other tests."""
import ctypes as C

import numpy as np
import pytest

from spined import lattices
from spined import _lib as L

pytestmark = pytest.mark.gpu

RTOL = 1e-11  # the tolerance of the FP64 expectation tests


def _call(lib, op, dtype, x, y, out):
    D, b = x.shape
    return lib.sed_operator_expectation_noalloc(op.ptr, dtype, D, b, C.c_void_p(x.data_ptr()), x.stride(1),
                                                C.c_void_p(y.data_ptr()), y.stride(1),
                                                C.c_void_p(out.ctypes.data))


@pytest.mark.parametrize("complex_model,form", [(False, L.SED_FORM_STREAM), (True, L.SED_FORM_ON_THE_FLY)])
def test_noalloc_matches_existing_entry_point(sed, complex_model, form):
    import torch
    from spined.model import build_model
    if complex_model:
        m = lattices.heisenberg_chain(16, momentum=3, parity=None, spin_inversion=None)
        dtype, tdt, ndt = 3, torch.complex128, np.complex128
    else:
        m = lattices.heisenberg_chain(20, j2=0.3)
        dtype, tdt, ndt = 1, torch.float64, np.float64
    built = build_model(m)
    op = built.hamiltonian
    op.prepare(form)  # the operator must be prepared before the no-allocation call
    D = sed.get_number_states(built.basis)
    lib = L.load()
    gen = torch.Generator(device="cuda").manual_seed(3)
    for call in range(2):  # two calls in a row share the scratch array
        x = torch.randn(3, D, dtype=tdt, device="cuda", generator=gen).t()  # column-major, stride D
        y = torch.zeros(3, D, dtype=tdt, device="cuda").t()
        out = np.zeros(3, dtype=np.complex128)
        st = _call(lib, op, dtype, x, y, out)
        assert st == 0, L.error_message(st)
        torch.cuda.synchronize()
        xh = np.asfortranarray(x.cpu().numpy().astype(ndt))
        want = sed.expectation(op, xh)  # existing entry point
        np.testing.assert_allclose(out, want, rtol=RTOL, atol=0)
        for c in range(3):
            yc = sed.apply(op, np.ascontiguousarray(xh[:, c]))
            np.testing.assert_allclose(y[:, c].cpu().numpy(), yc, rtol=0, atol=1e-12 * np.abs(yc).max())


def test_noalloc_rejects_what_it_cannot_do(sed):
    import torch
    from spined.model import build_model
    built = build_model(lattices.heisenberg_chain(12))
    op = built.hamiltonian
    D = sed.get_number_states(built.basis)
    lib = L.load()
    x = torch.randn(1, D, dtype=torch.float64, device="cuda").t()
    y = torch.zeros_like(x)
    out = np.zeros(1, dtype=np.complex128)
    assert _call(lib, op, 1, x, y, out) == L.LS_CACHE_NOT_BUILT  # not prepared: would have to allocate
    op.prepare(L.SED_FORM_STREAM)
    xb = torch.randn(65, D, dtype=torch.float64, device="cuda").t()
    yb = torch.zeros_like(xb)
    outb = np.zeros(65, dtype=np.complex128)
    st = _call(lib, op, 1, xb, yb, outb)
    assert st == L.LS_INVALID_ARGUMENT and "64 columns" in L.error_message(st)
    xh = np.zeros((D, 1))
    st = lib.sed_operator_expectation_noalloc(op.ptr, 1, D, 1, C.c_void_p(xh.ctypes.data), D,
                                              C.c_void_p(y.data_ptr()), D, C.c_void_p(out.ctypes.data))
    assert st == L.LS_INVALID_ARGUMENT  # host x: the caller owns device buffers
