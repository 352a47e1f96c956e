"""Failure paths of the C ABI, made on the host and checked through the
status convention of src/SpinED/Internal.hs:48-65 (a non-zero status whose
message comes from ls_error_to_string, raised by the host mirror as
LatticeSymmetriesException):

- the eigensolvers stop at max_iter with LS_NOT_CONVERGED;
- a caller-set cap on libsed's device memory makes allocations fail with
  LS_OUT_OF_MEMORY, as an exhausted cudaMalloc does;
- the batched persistent kernel's group barriers wait for arrivals that never
  come (a host-set test hook), their bounded waits run out after the
  caller-set limit, and the call fails with LS_DEVICE_TIMEOUT.

After each failure the same process solves normally again: no failure leaves
the CUDA context or libsed's state unusable. No GPU fault is involved."""
import time

import numpy as np
import pytest

from spined import lattices
from spined import _lib as L
from spined.model import build_model

pytestmark = pytest.mark.gpu


def test_max_iter_gives_not_converged(sed):
    built = build_model(lattices.heisenberg_chain(20, j2=0.2))
    op = built.hamiltonian
    for kw in ({}, {"max_basis": 8}, {"precision": L.SED_PRECISION_MIXED}):
        with pytest.raises(sed.LatticeSymmetriesException) as e:
            sed.eigh(op, tol=1e-8, max_iter=6, **kw)
        assert e.value.code == L.LS_NOT_CONVERGED, kw
        assert "did not converge" in str(e.value)
    with pytest.raises(sed.LatticeSymmetriesException) as e:
        sed.eigh_batched([op, build_model(lattices.heisenberg_chain(16)).hamiltonian], nev=2, max_iter=8)
    assert e.value.code == L.LS_NOT_CONVERGED
    r = sed.eigh(op, tol=1e-8)  # the same operator converges without the cap
    assert r.residuals[0] <= 1e-8


def test_device_memory_limit_gives_out_of_memory(sed):
    lib = L.load()
    lib.sed_release_workspace()
    m = lattices.heisenberg_chain(24)
    try:
        lib.sed_set_device_memory_limit(lib.sed_device_memory_in_use() + 16 * 1024)
        fresh = build_model(m, build=False)
        with pytest.raises(sed.LatticeSymmetriesException) as e:
            sed.build_basis(fresh.basis)
        assert e.value.code == L.LS_OUT_OF_MEMORY
        assert "device-memory limit" in str(e.value)
    finally:
        lib.sed_set_device_memory_limit(0)
    built = build_model(m)
    # a cap that the basis fits under but the Krylov workspace does not
    try:
        lib.sed_release_workspace()
        lib.sed_set_device_memory_limit(lib.sed_device_memory_in_use() + 64 * 1024)
        with pytest.raises(sed.LatticeSymmetriesException) as e:
            sed.eigh(built.hamiltonian, tol=1e-8)
        assert e.value.code == L.LS_OUT_OF_MEMORY
    finally:
        lib.sed_set_device_memory_limit(0)
    r = sed.eigh(built.hamiltonian, tol=1e-8)
    assert r.residuals[0] <= 1e-8


def test_batched_barrier_wait_runs_out(sed):
    lib = L.load()
    ops = [build_model(lattices.heisenberg_chain(n, j2=0.1)).hamiltonian for n in (16, 18, 20)]
    try:
        lib.sed_set_device_wait_limit(0.5)
        lib.sed_debug_barrier_extra_arrivals(1)
        t0 = time.perf_counter()
        with pytest.raises(sed.LatticeSymmetriesException) as e:
            sed.eigh_batched(ops, nev=2)
        waited = time.perf_counter() - t0
        assert e.value.code == L.LS_DEVICE_TIMEOUT
        assert "timed out" in str(e.value)
        assert waited < 30.0  # one bounded wait (0.5 s), not the 20 s default
    finally:
        lib.sed_debug_barrier_extra_arrivals(0)
        lib.sed_set_device_wait_limit(0.0)
    res = sed.eigh_batched(ops, nev=2)  # the context and the kernel still work
    assert np.all(res.residuals <= 1e-8)
    for i, op in enumerate(ops):
        r = sed.eigh(op, nev=2, tol=1e-8)
        np.testing.assert_allclose(res.eigenvalues[i], r.eigenvalues, rtol=1e-10)
