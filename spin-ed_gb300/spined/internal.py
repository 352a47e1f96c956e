"""Host mirror of src/SpinED/Internal.hs over libsed's C ABI.

Same names (snake_case), argument meanings, validation and exceptions as the
Haskell FFI shim, so that SpinED's own tests read the same against it:

    mkSymmetry     -> mk_symmetry       (Internal.hs:99-116)
    mkGroup        -> mk_group          (Internal.hs:141-150)
    mkBasis        -> mk_basis          (Internal.hs:199-228)
    buildBasis     -> build_basis       (Internal.hs:230-236)
    basisGetStates -> basis_get_states  (Internal.hs:238-244)
    getNumberStates-> get_number_states (Internal.hs:247-254)
    mkInteraction' -> mk_interaction    (Internal.hs:293-362)
    mkOperator     -> mk_operator       (Internal.hs:391-402)
    inplaceApply   -> inplace_apply     (Internal.hs:411-429)
    apply          -> apply             (Internal.hs:431-435)
    expectation    -> expectation       (Internal.hs:437-452)
    isOperatorReal'-> is_operator_real  (Internal.hs:454-455)
    PRIMME eigh    -> eigh              (src/SpinED.hs:404, via sed_eigh)

Vectors may be numpy arrays (host) or CUDA tensors exposing data_ptr()
(device); libsed detects which.
"""
from __future__ import annotations

import ctypes as C
import weakref
from dataclasses import dataclass
from typing import Sequence

import numpy as np

from . import _lib as L


class LatticeSymmetriesException(Exception):
    """A non-zero status from libsed (Internal.hs:28-32)."""

    def __init__(self, code: int, message: str):
        super().__init__(f"{message} (status {code})")
        self.code = code
        self.message = message


class SpinEDException(Exception):
    """Input rejected before reaching the library (Internal.hs:34-37)."""


def check_status(code: int) -> None:
    """Internal.hs:56-65."""
    if code != 0:
        raise LatticeSymmetriesException(code, L.error_message(code))


class _Handle:
    _destroy = ""

    def __init__(self, ptr: C.c_void_p):
        self._ptr = ptr

    @property
    def ptr(self) -> C.c_void_p:
        return self._ptr

    def __del__(self):
        p = getattr(self, "_ptr", None)
        if p and p.value and L._lib is not None:
            getattr(L._lib, self._destroy)(p)
            self._ptr = None


def _mk(fn, *args) -> C.c_void_p:
    out = C.c_void_p()
    check_status(fn(C.byref(out), *args))
    return out


# --------------------------------------------------------------- symmetry --
class Symmetry(_Handle):
    _destroy = "ls_destroy_symmetry"

    @property
    def sector(self) -> int:
        return L.load().ls_get_sector(self.ptr)

    @property
    def periodicity(self) -> int:
        return L.load().ls_get_periodicity(self.ptr)

    @property
    def phase(self) -> float:
        return L.load().ls_get_phase(self.ptr)


def mk_symmetry(permutation: Sequence[int], sector: int) -> Symmetry:
    """Internal.hs:99-116."""
    if any(p < 0 for p in permutation):
        raise SpinEDException(f"invalid permutation: {list(permutation)}; indices must be non-negative")
    if sector < 0:
        raise SpinEDException(f"invalid sector: {sector}; expected a non-negative number")
    p = np.ascontiguousarray(permutation, dtype=np.uint32)
    return Symmetry(_mk(L.load().ls_create_symmetry, len(p), C.c_void_p(p.ctypes.data), sector))


def get_sector(s: Symmetry) -> int:
    return s.sector


def get_periodicity(s: Symmetry) -> int:
    return s.periodicity


def get_phase(s: Symmetry) -> float:
    return s.phase


class SymmetryGroup(_Handle):
    _destroy = "ls_destroy_group"

    def __init__(self, ptr, generators):
        super().__init__(ptr)
        self._generators = list(generators)  # keep alive like withManyForeignPtr


def mk_group(symmetries: Sequence[Symmetry]) -> SymmetryGroup:
    """Internal.hs:141-150."""
    arr = (C.c_void_p * max(1, len(symmetries)))(*[s.ptr.value for s in symmetries])
    return SymmetryGroup(_mk(L.load().ls_create_group, len(symmetries), arr), symmetries)


def get_group_size(g: SymmetryGroup) -> int:
    return L.load().ls_get_group_size(g.ptr)


# ------------------------------------------------------------------ basis --
class SpinBasis(_Handle):
    _destroy = "ls_destroy_spin_basis"

    def __init__(self, ptr, group, number_spins, hamming_weight, spin_inversion):
        super().__init__(ptr)
        self.group = group
        self.number_spins = number_spins
        self.hamming_weight = hamming_weight
        self.spin_inversion = spin_inversion

    def state_info(self, bits: int) -> tuple[int, int, int]:
        rep, ph, mod = C.c_uint64(), C.c_uint(), C.c_uint()
        check_status(L.load().sed_basis_state_info(self.ptr, bits, C.byref(rep), C.byref(ph), C.byref(mod)))
        return rep.value, ph.value, mod.value

    def index(self, rep: int) -> int | None:
        out = C.c_uint64()
        st = L.load().sed_basis_index(self.ptr, rep, C.byref(out))
        if st == L.LS_NOT_A_REPRESENTATIVE:
            return None
        check_status(st)
        return out.value

    def norms(self) -> np.ndarray:
        out = np.zeros(get_number_states(self), dtype=np.float64)
        check_status(L.load().sed_basis_get_norms(self.ptr, C.c_void_p(out.ctypes.data)))
        return out


def mk_basis(group: SymmetryGroup, number_spins: int, hamming_weight: int | None = None,
             spin_inversion: int | None = None) -> SpinBasis:
    """Internal.hs:199-228."""
    if number_spins <= 0:
        raise SpinEDException(f"invalid number of spins: {number_spins}; expected a positive number")
    hw = -1
    if hamming_weight is not None:
        if hamming_weight < 0:
            raise SpinEDException(f"invalid Hamming weight: {hamming_weight}; expected a non-negative number")
        hw = hamming_weight
    inv = 0
    if spin_inversion is not None:
        if spin_inversion not in (1, -1):
            raise SpinEDException(f"invalid value for spin inversion: {spin_inversion}; expected either -1 or +1")
        inv = spin_inversion
    ptr = _mk(L.load().ls_create_spin_basis, group.ptr, number_spins, hw, inv)
    return SpinBasis(ptr, group, number_spins, hamming_weight, spin_inversion)


def build_basis(basis: SpinBasis, representatives: np.ndarray | None = None) -> None:
    """Internal.hs:230-236: ls_build, or ls_build_unsafe with a given list."""
    lib = L.load()
    if representatives is None:
        check_status(lib.ls_build(basis.ptr))
    else:
        v = np.ascontiguousarray(representatives, dtype=np.uint64)
        check_status(lib.ls_build_unsafe(basis.ptr, len(v), C.c_void_p(v.ctypes.data)))


def basis_get_states(basis: SpinBasis) -> np.ndarray:
    """Internal.hs:238-244: a view of the host copy owned by a states object,
    which is destroyed when the array (and every view of it) is collected,
    as the reference's ForeignPtr finaliser does."""
    lib = L.load()
    states = _mk(lib.ls_get_states, basis.ptr)
    n = lib.ls_states_get_size(states)
    if not n:
        lib.ls_destroy_states(states)
        return np.zeros(0, np.uint64)
    data = lib.ls_states_get_data(states)
    out = np.ctypeslib.as_array(C.cast(data, C.POINTER(C.c_uint64)), shape=(n,))
    weakref.finalize(out, lib.ls_destroy_states, states)
    return out


def get_number_states(basis: SpinBasis) -> int:
    """Internal.hs:247-254."""
    n = C.c_uint64()
    check_status(L.load().ls_get_number_states(basis.ptr, C.byref(n)))
    return n.value


# ------------------------------------------------------------ interaction --
class Interaction(_Handle):
    _destroy = "ls_destroy_interaction"


def _to_matrix(dim: int, rows) -> np.ndarray:
    """toMatrix (Internal.hs:278-291)."""
    rows = [list(r) for r in rows]
    if len(rows) != dim or any(len(r) != dim for r in rows):
        raise SpinEDException(f"invalid matrix: {rows}; expected a square matrix of dimension {dim}")
    m = np.zeros((dim, dim), dtype=np.complex128)
    for i, r in enumerate(rows):
        for j, v in enumerate(r):
            m[i, j] = complex(v[0], v[1]) if isinstance(v, (list, tuple)) else complex(v)
    return m


def mk_interaction(matrix, sites: Sequence[Sequence[int]]) -> Interaction:
    """mkInteraction' for [[Int]] sites (Internal.hs:324-362)."""
    sites = [list(s) for s in sites]
    if not sites:
        raise SpinEDException("zero-point interactions (i.e. constant factors) are not supported")
    n = len(sites[0])
    if n not in (1, 2, 3, 4):
        raise SpinEDException(f"currently only 1-, 2-, 3-, and 4-point interactions are supported, but received n={n}")
    if any(len(s) != n for s in sites):
        raise SpinEDException(f"invalid sites: {sites}; expected an array of length-{n} tuples")
    m = _to_matrix(2**n, matrix)
    if any(x < 0 for s in sites for x in s):
        raise SpinEDException("site indices must be all non-negative numbers")
    flat = np.ascontiguousarray(np.array(sites, dtype=np.uint16).ravel())
    mm = np.ascontiguousarray(m)
    fn = getattr(L.load(), f"ls_create_interaction{n}")
    ptr = _mk(fn, C.c_void_p(mm.ctypes.data), len(sites), C.c_void_p(flat.ctypes.data))
    return Interaction(ptr)


def is_real_interaction(x: Interaction) -> bool:
    return bool(L.load().ls_interaction_is_real(x.ptr))


# --------------------------------------------------------------- operator --
class Operator(_Handle):
    _destroy = "ls_destroy_operator"

    def __init__(self, ptr, basis, terms):
        super().__init__(ptr)
        self.basis = basis
        self._terms = list(terms)

    def prepare(self, form: int = L.SED_FORM_STREAM) -> None:
        check_status(L.load().sed_operator_prepare(self.ptr, form))

    @property
    def stream_bytes(self) -> int:
        return L.load().sed_operator_stream_bytes(self.ptr)

    @property
    def stream_elements(self) -> int:
        return L.load().sed_operator_stream_elements(self.ptr)


def mk_operator(basis: SpinBasis, terms: Sequence[Interaction]) -> Operator:
    """Internal.hs:391-402."""
    arr = (C.c_void_p * max(1, len(terms)))(*[t.ptr.value for t in terms])
    return Operator(_mk(L.load().ls_create_operator, basis.ptr, len(terms), arr), basis, terms)


def is_operator_real(op: Operator) -> bool:
    return bool(L.load().ls_operator_is_real(op.ptr))


_DTYPES = {np.dtype(np.float32): 0, np.dtype(np.float64): 1, np.dtype(np.complex64): 2,
           np.dtype(np.complex128): 3}
_TORCH_DTYPES = {"torch.float32": 0, "torch.float64": 1, "torch.complex64": 2, "torch.complex128": 3}


def _block(a):
    """(pointer, dtype code, size, block, stride) of a column-major block."""
    if isinstance(a, np.ndarray):
        code = _DTYPES.get(a.dtype)
        if code is None:
            raise SpinEDException(f"unsupported dtype {a.dtype}")
        if a.ndim == 1:
            return C.c_void_p(a.ctypes.data), code, a.shape[0], 1, a.shape[0]
        if a.strides[0] != a.itemsize:
            raise SpinEDException("blocks must be column-major (Fortran order)")
        return C.c_void_p(a.ctypes.data), code, a.shape[0], a.shape[1], a.strides[1] // a.itemsize
    # torch tensor (device or host)
    code = _TORCH_DTYPES.get(str(a.dtype))
    if code is None:
        raise SpinEDException(f"unsupported dtype {a.dtype}")
    if a.dim() == 1:
        return C.c_void_p(a.data_ptr()), code, a.shape[0], 1, a.shape[0]
    if a.stride(0) != 1:
        raise SpinEDException("blocks must be column-major")
    return C.c_void_p(a.data_ptr()), code, a.shape[0], a.shape[1], a.stride(1)


def inplace_apply(op: Operator, x, y) -> None:
    """Internal.hs:411-429: y <- H x."""
    px, cx, nx, bx, sx = _block(x)
    py, cy, ny, by, sy = _block(y)
    if (nx, bx) != (ny, by):
        raise SpinEDException(f"dimensions of x and y do not match: {(nx, bx)} != {(ny, by)}")
    if cx != cy:
        raise SpinEDException("x and y have different dtypes")
    check_status(L.load().ls_operator_matmat(op.ptr, cx, nx, bx, px, sx, py, sy))


def apply(op: Operator, x):
    """Internal.hs:431-435."""
    if isinstance(x, np.ndarray):
        y = np.zeros_like(x, order="F")
    else:
        y = x.new_zeros(x.shape) if x.dim() == 1 else x.new_zeros(x.shape[1], x.shape[0]).t()
    inplace_apply(op, x, y)
    return y


def expectation(op: Operator, x) -> np.ndarray:
    """Internal.hs:437-452: <x_c|H|x_c> per column (complex128)."""
    px, cx, n, b, s = _block(x)
    out = np.zeros(b, dtype=np.complex128)
    check_status(L.load().ls_operator_expectation(op.ptr, cx, n, b, px, s, C.c_void_p(out.ctypes.data)))
    return out


@dataclass
class EighResult:
    eigenvalues: np.ndarray
    eigenvectors: np.ndarray
    residuals: np.ndarray
    iterations: int
    matvecs: int
    restarts: int
    fp32_iterations: int
    seconds_total: float
    seconds_setup: float
    seconds_solve: float


def eigh_options(nev: int = 1, tol: float = 1e-8, max_iter: int = 0, max_basis: int = 0,
                 block_size: int = 1, precision: int = L.SED_PRECISION_FP64, seed: int = 1234,
                 start=None, form: int = L.SED_FORM_AUTO) -> tuple[L.EighOptions, object]:
    opts = L.EighOptions()
    L.load().sed_eigh_options_init(C.byref(opts))
    opts.nev, opts.tol, opts.max_iter, opts.max_basis = nev, tol, max_iter, max_basis
    opts.block_size, opts.precision, opts.seed, opts.form = block_size, precision, seed, form
    keep = None
    if start is not None:
        if isinstance(start, np.ndarray):
            keep = np.asfortranarray(start, dtype=np.float64)
            ptr, _, n, b, s = _block(keep)
        else:
            keep = start
            ptr, _, n, b, s = _block(start)
        opts.start = L.SED_START_GIVEN
        opts.start_vectors = ptr
        opts.start_stride = s
    return opts, keep


def eigh(op: Operator, nev: int = 1, tol: float = 1e-8, dtype=np.float64, out=None,
         **kw) -> EighResult:
    """Lowest eigenpairs through sed_eigh (replaces Numeric.PRIMME.eigh, src/SpinED.hs:404)."""
    D = get_number_states(op.basis)
    opts, keep = eigh_options(nev=nev, tol=tol, **kw)
    evals = np.zeros(nev, dtype=np.float64)
    res = np.zeros(nev, dtype=np.float64)
    if out is None:
        out = np.zeros((D, nev), dtype=dtype, order="F")
    pv, code, n, b, s = _block(out)
    info = L.EighInfo()
    check_status(L.load().sed_eigh(op.ptr, code, C.byref(opts), C.c_void_p(evals.ctypes.data), pv, s,
                                   C.c_void_p(res.ctypes.data), C.byref(info)))
    del keep
    return EighResult(evals, out, res, info.iterations, info.matvecs, info.restarts, info.fp32_iterations,
                      info.seconds_total, info.seconds_setup, info.seconds_solve)


@dataclass
class BatchResult:
    eigenvalues: np.ndarray      # [count, nev]
    residuals: np.ndarray        # [count, nev]
    eigenvectors: list           # per operator [D_i, nev] (or None)
    block_steps_max: int
    restarts_max: int
    kernel_ms: float
    seconds_total: float
    seconds_setup: float
    ctas_per_sm: int
    grid: int


def eigh_batched(ops: Sequence[Operator], nev: int = 4, tol: float = 1e-8, max_basis: int = 0,
                 seed: int = 1234, max_iter: int = 0, vectors: bool = True) -> BatchResult:
    """Lowest nev (<= 4) eigenpairs of every operator by block Lanczos (block
    size 4; FP64 vectors and matvec, double-float Gram-Schmidt products), all
    operators in one persistent launch (sed_eigh_batched)."""
    count = len(ops)
    opts, _ = eigh_options(nev=nev, tol=tol, max_iter=max_iter, max_basis=max_basis, block_size=4, seed=seed)
    evals = np.zeros((count, nev), dtype=np.float64)
    res = np.zeros((count, nev), dtype=np.float64)
    arr = (C.c_void_p * count)(*[op.ptr.value for op in ops])
    vecs, vptr, lds = None, None, None
    if vectors:
        vecs = [np.zeros((get_number_states(op.basis), nev), dtype=np.float64, order="F") for op in ops]
        vptr = (C.c_void_p * count)(*[v.ctypes.data for v in vecs])
        lds = (C.c_uint64 * count)(*[v.shape[0] for v in vecs])
    info = L.BatchInfo()
    check_status(L.load().sed_eigh_batched(count, C.cast(arr, C.c_void_p), C.byref(opts),
                                           C.c_void_p(evals.ctypes.data), C.c_void_p(res.ctypes.data),
                                           C.cast(vptr, C.c_void_p) if vptr is not None else None,
                                           C.cast(lds, C.c_void_p) if lds is not None else None,
                                           C.byref(info)))
    return BatchResult(evals, res, vecs, info.block_steps_max, info.restarts_max, info.kernel_ms,
                       info.seconds_total, info.seconds_setup, info.ctas_per_sm, info.grid)
