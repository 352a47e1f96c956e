"""Python face of the CPU oracle (oracle.c).

TEST INFRASTRUCTURE ONLY. The parity tests, ``__graft_entry__.smoke()`` and
the CPU-baseline leg of ``bench.py`` import this module to obtain expected
values; no product code path imports it.

The C library restates the arithmetic that the reference delegates to
lattice-symmetries (``src/SpinED/Internal.hs:67-458``); this module adds the
eigensolver restatement the reference takes from PRIMME
(``src/SpinED.hs:370-411``): a plain FP64 Lanczos with full
re-orthogonalisation, used as the FP64 oracle for eigenvalues.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass
from typing import Sequence

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")

OR_OK = 0
OR_INVALID_PERMUTATION = 10
OR_INVALID_SECTOR = 11
OR_INCOMPATIBLE_SYMMETRIES = 12
OR_GROUP_TOO_BIG = 13
OR_INVALID_ARGUMENT = 14


class OracleError(RuntimeError):
    def __init__(self, code: int, what: str):
        super().__init__(f"oracle error {code} in {what}")
        self.code = code


def build(force: bool = False) -> str:
    """Compile oracle.c with gcc + OpenMP into oracle/_build/liboracle.so."""
    src = os.path.join(HERE, "oracle.c")
    if not force and os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= max(
        os.path.getmtime(src), os.path.getmtime(os.path.join(HERE, "oracle.h"))
    ):
        return LIB_PATH
    os.makedirs(os.path.dirname(LIB_PATH), exist_ok=True)
    tmp = LIB_PATH + f".tmp{os.getpid()}"
    subprocess.check_call(
        ["gcc", "-std=c11", "-O2", "-fopenmp", "-fPIC", "-shared", "-o", tmp, src, "-lm"]
    )
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        u, i, u64, p = C.c_uint, C.c_int, C.c_uint64, C.c_void_p
        L.or_symmetry_info.argtypes = [u, p, u, C.POINTER(u)]
        L.or_group_closure.argtypes = [u, u, p, p, u, p, p, C.POINTER(u), C.POINTER(u)]
        L.or_basis_create.argtypes = [C.POINTER(p), u, i, i, u, p, p, u]
        L.or_basis_destroy.argtypes = [p]
        L.or_apply.argtypes = [p, u, u64]
        L.or_apply.restype = u64
        L.or_representative_weight.argtypes = [p, u64]
        L.or_representative_weight.restype = u
        L.or_state_info.argtypes = [p, u64, C.POINTER(u), C.POINTER(i)]
        L.or_state_info.restype = u64
        L.or_enumerate.argtypes = [p, u64, u64, p, p, u64, C.POINTER(u64)]
        L.or_space_size.argtypes = [p]
        L.or_space_size.restype = u64
        L.or_operator_create.argtypes = [C.POINTER(p), p, u, p, p, p, p]
        L.or_operator_destroy.argtypes = [p]
        L.or_matvec.argtypes = [p, u64, p, p, p, p, u64, u64]
        L.or_matvec_rows.argtypes = [p, u64, p, p, p, p, u64, u64]
        L.or_matrix_coo.argtypes = [p, u64, p, p, p, p, p, u64, C.POINTER(u64)]
        L.or_row_work.argtypes = [p, p, u64, C.POINTER(u64)]
        L.or_row_work.restype = u64
        L.or_philox4x32_10.argtypes = [p, p, p]
        L.or_start_vector.argtypes = [u64, u64, p]
        L.or_num_threads.restype = i
        _lib = L
    return _lib


def _ptr(a: np.ndarray) -> C.c_void_p:
    return C.c_void_p(a.ctypes.data)


def symmetry_info(perm: Sequence[int], sector: int) -> int:
    """Periodicity of ``perm``; raises OracleError on invalid input."""
    p = np.ascontiguousarray(perm, dtype=np.uint32)
    per = C.c_uint(0)
    st = lib().or_symmetry_info(len(p), _ptr(p), sector, C.byref(per))
    if st:
        raise OracleError(st, "symmetry")
    return per.value


@dataclass
class Group:
    n: int
    perms: np.ndarray  # [G, n] uint32
    phases: np.ndarray  # [G] uint32 (numerators mod L)
    L: int

    @property
    def size(self) -> int:
        return len(self.perms)


def group_closure(n: int, generators: Sequence[tuple[Sequence[int], int]], max_size: int = 65536) -> Group:
    """Closure of (permutation, sector) generators (src/SpinED/Internal.hs:141-150)."""
    g = len(generators)
    perms = np.ascontiguousarray([p for p, _ in generators], dtype=np.uint32).reshape(g, n)
    sectors = np.ascontiguousarray([s for _, s in generators], dtype=np.uint32)
    out_p = np.zeros((max_size, n), dtype=np.uint32)
    out_ph = np.zeros(max_size, dtype=np.uint32)
    L, size = C.c_uint(0), C.c_uint(0)
    st = lib().or_group_closure(g, n, _ptr(perms), _ptr(sectors), max_size, _ptr(out_p), _ptr(out_ph),
                                C.byref(L), C.byref(size))
    if st:
        raise OracleError(st, "group")
    return Group(n, out_p[: size.value].copy(), out_ph[: size.value].copy(), L.value)


class Basis:
    """Symmetry-adapted spin basis (src/SpinED/Internal.hs:199-236)."""

    def __init__(self, n: int, hamming_weight: int | None, spin_inversion: int | None,
                 generators: Sequence[tuple[Sequence[int], int]] = ()):
        self.n = n
        self.hw = -1 if hamming_weight is None else hamming_weight
        self.inv = 0 if spin_inversion is None else spin_inversion
        self.group = group_closure(n, list(generators)) if generators else Group(
            n, np.arange(n, dtype=np.uint32)[None, :], np.zeros(1, dtype=np.uint32), 1)
        h = C.c_void_p()
        st = lib().or_basis_create(C.byref(h), n, self.hw, self.inv, self.group.size,
                                   _ptr(self.group.perms), _ptr(self.group.phases), self.group.L)
        if st:
            raise OracleError(st, "basis")
        self._h = h
        self.reps: np.ndarray | None = None
        self.weights: np.ndarray | None = None

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.or_basis_destroy(self._h)
            self._h = None

    @property
    def group_order(self) -> int:
        """|G| counting spin inversion."""
        return self.group.size * (2 if self.inv else 1)

    def space_size(self) -> int:
        return lib().or_space_size(self._h)

    def count(self, rank_begin: int = 0, rank_end: int = 2**64 - 1) -> int:
        n = C.c_uint64(0)
        st = lib().or_enumerate(self._h, rank_begin, rank_end, None, None, 0, C.byref(n))
        if st:
            raise OracleError(st, "enumerate")
        return n.value

    def build(self, rank_begin: int = 0, rank_end: int = 2**64 - 1) -> np.ndarray:
        """Enumerate representatives (ls_build, src/SpinED/Internal.hs:178-179)."""
        D = self.count(rank_begin, rank_end)
        reps = np.zeros(max(D, 1), dtype=np.uint64)
        w = np.zeros(max(D, 1), dtype=np.uint32)
        n = C.c_uint64(0)
        st = lib().or_enumerate(self._h, rank_begin, rank_end, _ptr(reps), _ptr(w), D, C.byref(n))
        if st:
            raise OracleError(st, "enumerate")
        self.reps, self.weights = reps[:D], w[:D]
        return self.reps

    def slice(self, rank_begin: int, rank_end: int) -> tuple[np.ndarray, np.ndarray]:
        """Representatives and stabiliser orders of the word ranks
        [rank_begin, rank_end), without replacing the built list."""
        saved = self.reps, self.weights
        try:
            reps = self.build(rank_begin, rank_end)
            return reps.copy(), self.weights.copy()
        finally:
            self.reps, self.weights = saved

    def norms(self) -> np.ndarray:
        """||P r|| = sqrt(S / |G|) per representative."""
        return np.sqrt(self.weights.astype(np.float64) / float(self.group_order))

    def apply(self, g: int, x: int) -> int:
        return lib().or_apply(self._h, g, x)

    def representative_weight(self, x: int) -> int:
        return lib().or_representative_weight(self._h, x)

    def state_info(self, x: int) -> tuple[int, int, bool]:
        ph, inv = C.c_uint(0), C.c_int(0)
        r = lib().or_state_info(self._h, x, C.byref(ph), C.byref(inv))
        return r, ph.value, bool(inv.value)


@dataclass
class Term:
    """One interaction: a 2^k x 2^k matrix applied to k-site tuples."""
    matrix: np.ndarray  # complex128 [2^k, 2^k]
    sites: np.ndarray  # int [T, k]

    @property
    def k(self) -> int:
        return self.sites.shape[1]


class Operator:
    """Operator in the symmetry-adapted basis (src/SpinED/Internal.hs:391-429)."""

    def __init__(self, basis: Basis, terms: Sequence[Term], build: bool = True):
        if basis.reps is None and build:
            basis.build()
        self.basis = basis
        ks = np.array([t.k for t in terms], dtype=np.uint32)
        nt = np.array([len(t.sites) for t in terms], dtype=np.uint32)
        mats = np.concatenate([np.asarray(t.matrix, dtype=np.complex128).ravel() for t in terms]) if terms else np.zeros(1, np.complex128)
        mats = np.ascontiguousarray(mats).view(np.float64)
        sites = np.concatenate([np.asarray(t.sites, dtype=np.uint16).ravel() for t in terms]) if terms else np.zeros(1, np.uint16)
        sites = np.ascontiguousarray(sites, dtype=np.uint16)
        self._keep = (ks, nt, mats, sites)
        h = C.c_void_p()
        st = lib().or_operator_create(C.byref(h), basis._h, len(terms), _ptr(ks), _ptr(nt), _ptr(mats), _ptr(sites))
        if st:
            raise OracleError(st, "operator")
        self._h = h
        self.is_real = all(np.all(np.imag(t.matrix) == 0) for t in terms) and _real_characters(basis)

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.or_operator_destroy(self._h)
            self._h = None

    @property
    def dim(self) -> int:
        return 0 if self.basis.reps is None else len(self.basis.reps)

    def row_work(self, rows: np.ndarray) -> int:
        """Element generation + canonicalisation for `rows` (no lookup); returns the element count."""
        r = np.ascontiguousarray(rows, dtype=np.uint64)
        n = C.c_uint64(0)
        lib().or_row_work(self._h, _ptr(r), len(r), C.byref(n))
        return n.value

    def matvec(self, x: np.ndarray, row_begin: int = 0, row_end: int | None = None) -> np.ndarray:
        x = np.ascontiguousarray(x, dtype=np.complex128)
        y = np.zeros(self.dim, dtype=np.complex128)
        re = self.dim if row_end is None else row_end
        b = self.basis
        lib().or_matvec(self._h, self.dim, _ptr(b.reps), _ptr(b.weights), _ptr(x.view(np.float64)),
                        _ptr(y.view(np.float64)), row_begin, re)
        return y

    def matvec_rows(self, reps: np.ndarray, weights: np.ndarray, x: np.ndarray, row_begin: int,
                    row_end: int) -> np.ndarray:
        """Rows [row_begin, row_end) of H x over a representative list given
        by the caller (sorted, with stabiliser orders): the pull form of
        src/SpinED/Internal.hs:411-429, index lookups into `reps` included."""
        reps = np.ascontiguousarray(reps, dtype=np.uint64)
        weights = np.ascontiguousarray(weights, dtype=np.uint32)
        x = np.ascontiguousarray(x, dtype=np.complex128)
        D = len(reps)
        row_end = min(row_end, D)
        y = np.zeros(max(row_end - row_begin, 1), dtype=np.complex128)
        st = lib().or_matvec_rows(self._h, D, _ptr(reps), _ptr(weights), _ptr(x.view(np.float64)),
                                  _ptr(y.view(np.float64)), row_begin, row_end)
        if st:
            raise OracleError(st, "matvec_rows")
        return y[:max(row_end - row_begin, 0)]

    def coo(self):
        b = self.basis
        n = C.c_uint64(0)
        lib().or_matrix_coo(self._h, self.dim, _ptr(b.reps), _ptr(b.weights), None, None, None, 0, C.byref(n))
        nnz = n.value
        rows = np.zeros(max(nnz, 1), np.uint64)
        cols = np.zeros(max(nnz, 1), np.uint64)
        vals = np.zeros(max(nnz, 1), np.complex128)
        lib().or_matrix_coo(self._h, self.dim, _ptr(b.reps), _ptr(b.weights), _ptr(rows), _ptr(cols),
                            _ptr(vals.view(np.float64)), nnz, C.byref(n))
        return rows[:nnz], cols[:nnz], vals[:nnz]

    def sparse(self):
        import scipy.sparse as sp
        r, c, v = self.coo()
        if self.is_real:
            v = v.real
        return sp.csr_matrix((v, (r.astype(np.int64), c.astype(np.int64))), shape=(self.dim, self.dim))

    def dense(self) -> np.ndarray:
        return self.sparse().toarray()


def _real_characters(basis: Basis) -> bool:
    L = basis.group.L * (2 if (basis.inv == -1 and basis.group.L % 2) else 1)
    scale = L // basis.group.L
    ph = (basis.group.phases.astype(np.int64) * scale) % L
    return bool(np.all((2 * ph) % L == 0))


def philox4x32_10(ctr: Sequence[int], key: Sequence[int]) -> tuple[int, int, int, int]:
    c = np.ascontiguousarray(ctr, dtype=np.uint32)
    k = np.ascontiguousarray(key, dtype=np.uint32)
    out = np.zeros(4, dtype=np.uint32)
    lib().or_philox4x32_10(_ptr(c), _ptr(k), _ptr(out))
    return tuple(int(v) for v in out)


def start_vector(seed: int, D: int) -> np.ndarray:
    out = np.zeros(max(D, 1), dtype=np.float64)
    lib().or_start_vector(seed, D, _ptr(out))
    return out[:D]


def num_threads() -> int:
    return lib().or_num_threads()


def lanczos_ground_state(matvec, v0: np.ndarray, tol: float = 1e-8, max_iter: int = 500,
                         nev: int = 1):
    """Plain FP64 Lanczos with full re-orthogonalisation (the FP64 oracle).

    Returns (eigenvalues[nev], eigenvectors [D, nev], residual norms, iterations).
    Residual is ||H psi - E psi|| of the normalised Ritz vector.
    """
    dtype = np.result_type(v0.dtype, np.float64)
    D = len(v0)
    V = np.zeros((min(max_iter, D) + 1, D), dtype=dtype)
    V[0] = v0 / np.linalg.norm(v0)
    alpha, beta = [], []
    for k in range(min(max_iter, D)):
        w = matvec(V[k])
        a = np.vdot(V[k], w).real
        w = w - a * V[k] - (beta[-1] * V[k - 1] if k else 0)
        for _ in range(2):
            w = w - V[: k + 1].T @ (V[: k + 1].conj() @ w)
        b = np.linalg.norm(w)
        alpha.append(a)
        beta.append(b)
        m = k + 1
        if m >= nev and (m % 5 == 0 or b < 1e-12 or m == min(max_iter, D)):
            T = np.diag(alpha) + np.diag(beta[:-1], 1) + np.diag(beta[:-1], -1)
            ev, S = np.linalg.eigh(T)
            est = np.abs(b * S[-1, :nev])
            if np.all(est < tol * 0.1) or b < 1e-12 or m == min(max_iter, D):
                psi = V[:m].T @ S[:, :nev]
                psi /= np.linalg.norm(psi, axis=0)
                res = []
                evals = []
                for c in range(nev):
                    hp = matvec(psi[:, c])
                    e = np.vdot(psi[:, c], hp).real
                    evals.append(e)
                    res.append(np.linalg.norm(hp - e * psi[:, c]))
                if max(res) <= tol or b < 1e-12 or m == min(max_iter, D):
                    return np.array(evals), psi, np.array(res), m
        if b < 1e-300:
            break
        V[k + 1] = w / b
    raise RuntimeError("oracle Lanczos did not converge")
