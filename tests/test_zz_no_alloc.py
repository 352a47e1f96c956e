"""sed_operator_expectation_noalloc: the expectation entry point for callers
that cannot let a library allocate device memory (their device memory belongs
to their own pool allocator, or cudaMalloc's implicit synchronisation is too
costly for them). Called through the C ABI and checked against the existing
ls_operator_expectation / ls_operator_matmat on two calls in a row, in all
four dtypes and both matvec forms.

x and y are written by torch on its current stream, and that stream is the
one handed to the entry point, so the matvec is ordered after those writes.

This file is collected last on purpose; it passes alone in a fresh process
and after the other tests."""
import ctypes as C

import numpy as np
import pytest

from spined import lattices
from spined import _lib as L

pytestmark = pytest.mark.gpu

# the tolerances of the expectation and matvec tests: FP64 paths differ from
# the existing entry point only by summation order; FP32 paths by FP32
# rounding of the same sums
RTOL = {0: 2e-5, 1: 1e-11, 2: 2e-5, 3: 1e-11}
ATOL_Y = {0: 2e-5, 1: 1e-12, 2: 2e-5, 3: 1e-12}


def _call(lib, op, dtype, x, y, out, stream):
    D, b = x.shape
    return lib.sed_operator_expectation_noalloc(op.ptr, dtype, D, b, C.c_void_p(x.data_ptr()), x.stride(1),
                                                C.c_void_p(y.data_ptr()), y.stride(1),
                                                C.c_void_p(out.ctypes.data), C.c_void_p(stream))


@pytest.mark.parametrize("form", [L.SED_FORM_STREAM, L.SED_FORM_ON_THE_FLY])
@pytest.mark.parametrize("dtype", [0, 1, 2, 3])
def test_noalloc_matches_existing_entry_point(sed, dtype, form):
    import torch
    from spined.model import build_model
    if dtype >= 2:  # complex vectors on a complex operator (momentum sector)
        m = lattices.heisenberg_chain(16, momentum=3, parity=None, spin_inversion=None)
    else:
        m = lattices.heisenberg_chain(20, j2=0.3)
    tdt = {0: torch.float32, 1: torch.float64, 2: torch.complex64, 3: torch.complex128}[dtype]
    ndt = {0: np.float32, 1: np.float64, 2: np.complex64, 3: np.complex128}[dtype]
    built = build_model(m)
    op = built.hamiltonian
    op.prepare(form)  # the operator must be prepared before the no-allocation call
    D = sed.get_number_states(built.basis)
    lib = L.load()
    gen = torch.Generator(device="cuda").manual_seed(3)
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):  # two calls in a row share the scratch array
        x = torch.randn(3, D, dtype=tdt, device="cuda", generator=gen).t()  # column-major, stride D
        y = torch.zeros(3, D, dtype=tdt, device="cuda").t()
        out = np.zeros(3, dtype=np.complex128)
        st = _call(lib, op, dtype, x, y, out, stream)
        assert st == 0, L.error_message(st)
        xh = np.asfortranarray(x.cpu().numpy().astype(ndt))
        want = sed.expectation(op, xh)  # existing entry point
        np.testing.assert_allclose(out, want, rtol=RTOL[dtype], atol=0)
        for c in range(3):
            yc = sed.apply(op, np.ascontiguousarray(xh[:, c]))
            np.testing.assert_allclose(y[:, c].cpu().numpy(), yc, rtol=0,
                                       atol=ATOL_Y[dtype] * np.abs(yc).max())


def test_noalloc_rejects_what_it_cannot_do(sed):
    import torch
    from spined.model import build_model
    built = build_model(lattices.heisenberg_chain(12))
    op = built.hamiltonian
    D = sed.get_number_states(built.basis)
    lib = L.load()
    stream = torch.cuda.current_stream().cuda_stream
    x = torch.randn(1, D, dtype=torch.float64, device="cuda").t()
    y = torch.zeros_like(x)
    out = np.zeros(1, dtype=np.complex128)
    assert _call(lib, op, 1, x, y, out, stream) == L.LS_CACHE_NOT_BUILT  # not prepared: would have to allocate
    op.prepare(L.SED_FORM_STREAM)
    xb = torch.randn(65, D, dtype=torch.float64, device="cuda").t()
    yb = torch.zeros_like(xb)
    outb = np.zeros(65, dtype=np.complex128)
    st = _call(lib, op, 1, xb, yb, outb, stream)
    assert st == L.LS_INVALID_ARGUMENT and "64 columns" in L.error_message(st)
    xh = np.zeros((D, 1))
    st = lib.sed_operator_expectation_noalloc(op.ptr, 1, D, 1, C.c_void_p(xh.ctypes.data), D,
                                              C.c_void_p(y.data_ptr()), D, C.c_void_p(out.ctypes.data),
                                              C.c_void_p(stream))
    assert st == L.LS_INVALID_ARGUMENT  # host x: the caller owns device buffers
    # NULL stream: the operator's own stream, after the caller has finished x
    torch.cuda.synchronize()
    st = _call(lib, op, 1, x, y, out, 0)
    assert st == 0, L.error_message(st)
    want = sed.expectation(op, np.asfortranarray(x.cpu().numpy()))
    np.testing.assert_allclose(out, want, rtol=RTOL[1], atol=0)
