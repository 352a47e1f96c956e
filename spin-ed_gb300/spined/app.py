"""The YAML-in / HDF5-out driver: SpinED's runApp (app/Main.hs) on libsed.

Steps, as in the reference:
  readConfig -> toConfig           (src/SpinED.hs:252-261, 175-200)
  prepareOutputFile                (SpinED.hs:283-288): groups /basis,
                                   /hamiltonian, /observables, /_workspace
  buildRepresentatives             (SpinED.hs:315-337): load
                                   /basis/representatives when present
                                   (resume, ls_build_unsafe), else ls_build
                                   and write them
  diagonalize                      (SpinED.hs:370-411): sed_eigh in place of
                                   PRIMME; writes /hamiltonian/eigenvalues,
                                   eigenvectors, residuals
  computeExpectations              (SpinED.hs:296-313): <v|O|v> per
                                   observable into /observables/<name>

Choices where the reference delegates to PRIMME or leaves a gap:
* ``precision: 0`` (the default) means a residual tolerance of 1e-8;
* eigenvectors are written with shape (number_vectors, D), row c holding
  eigenvector c, which is what the reference's Block instance produces
  (SpinED.hs:362-368: a column-major D x n block viewed as an n x D row-major
  matrix);
* an existing /hamiltonian/eigenvectors of matching size is used as the start
  vector (warm start), unless ``warm_start=False``;
* max_primme_basis_size, max_primme_block_size and min_primme_restart_size
  tune PRIMME's Davidson iteration, which sed_eigh replaces; they are read
  and validated but do not change the Lanczos run (its stored-vector count
  is chosen from the dimension);
* ``datatype: float32`` stores eigenvectors as float32/complex64; the
  eigensolver itself always runs in FP64 (or FP32-stored mixed precision when
  asked for), so results are never less accurate than the FP64 path.
"""
from __future__ import annotations

import logging
import os
import time
from dataclasses import dataclass

import numpy as np

from . import _lib as L
from . import hdf5
from . import internal as I
from .config import ConfigSpec, read_config

log = logging.getLogger("spined")

BASIS_PATH, HAMILTONIAN_PATH, OBSERVABLES_PATH, WORKSPACE_PATH = "/basis", "/hamiltonian", "/observables", "/_workspace"


@dataclass
class Environment:
    config: ConfigSpec
    basis: I.SpinBasis
    group: I.SymmetryGroup
    hamiltonian: I.Operator
    observables: list  # (name, Operator)
    keep: list         # interactions and symmetries kept alive


def to_environment(cfg: ConfigSpec) -> Environment:
    """toConfig: symmetries -> group -> basis, terms -> operators (SpinED.hs:175-200)."""
    b = cfg.basis
    if b.number_spins > 64:
        raise I.SpinEDException(
            f"invalid number_spins: {b.number_spins}; exact diagonalization is not feasible "
            "for systems larger than 64 spins")
    syms = [I.mk_symmetry(s.permutation, s.sector) for s in b.symmetries]
    group = I.mk_group(syms)
    log.info("Symmetry group contains %d elements", I.get_group_size(group))
    basis = I.mk_basis(group, b.number_spins, b.hamming_weight, b.spin_inversion)
    keep = list(syms)

    def operator(spec):
        terms = [I.mk_interaction([[(z.real, z.imag) for z in row] for row in t.matrix], t.sites) for t in spec.terms]
        keep.extend(terms)
        return I.mk_operator(basis, terms)

    ham = operator(cfg.hamiltonian)
    obs = [(o.name, operator(o)) for o in cfg.observables]
    return Environment(cfg, basis, group, ham, obs, keep)


def _load(path: str) -> hdf5.Group:
    if os.path.exists(path) and os.path.getsize(path) > 0:
        return hdf5.read(path)
    return hdf5.Group()


def _save(path: str, root: hdf5.Group) -> None:
    d = os.path.dirname(os.path.abspath(path))
    os.makedirs(d, exist_ok=True)
    hdf5.write(path, root)


def prepare_output_file(env: Environment) -> hdf5.Group:
    root = _load(env.config.output)
    for p in (BASIS_PATH, HAMILTONIAN_PATH, OBSERVABLES_PATH, WORKSPACE_PATH):
        root.require(p)
    _save(env.config.output, root)
    return root


def build_representatives(env: Environment, root: hdf5.Group) -> None:
    reps = root.get_path(BASIS_PATH + "/representatives")
    if reps is not None:
        log.info("Loading representatives from %s/representatives...", BASIS_PATH)
        I.build_basis(env.basis, np.asarray(reps, dtype=np.uint64))
    else:
        log.info("Building a list of representatives...")
        I.build_basis(env.basis)
    log.info("Hilbert space dimension is %d", I.get_number_states(env.basis))
    if reps is None:
        root.require(BASIS_PATH)["representatives"] = I.basis_get_states(env.basis)
        _save(env.config.output, root)


def _overwrite(group: hdf5.Group, name: str, value, prefix: str) -> None:
    if name in group:
        log.warning("Overwriting %s/%s...", prefix, name)
    group[name] = value


def diagonalize(env: Environment, root: hdf5.Group, warm_start: bool = True, precision: int = L.SED_PRECISION_FP64):
    cfg = env.config
    D = I.get_number_states(env.basis)
    nev = cfg.number_vectors
    if nev < 1 or nev > D:
        raise I.SpinEDException(f"invalid number_vectors: {nev}; expected 1..{D}")
    is_real = I.is_operator_real(env.hamiltonian)
    tol = cfg.precision if cfg.precision > 0 else 1e-8
    start = None
    old = root.get_path(HAMILTONIAN_PATH + "/eigenvectors")
    if warm_start and old is not None and old.ndim == 2 and old.shape[1] == D:
        v = np.asarray(old, dtype=np.complex128 if np.iscomplexobj(old) else np.float64).sum(axis=0)
        if not is_real:
            v = v.astype(np.complex128)
        elif np.iscomplexobj(v):
            v = v.real.copy()
        nrm = np.linalg.norm(v)
        if nrm > 0:
            start = v / nrm
            log.info("Starting from the stored eigenvectors (warm start)")
    out_dtype = np.float64 if is_real else np.complex128
    log.info("Diagonalizing %s...", cfg.hamiltonian.name)
    t0 = time.perf_counter()
    res = I.eigh(env.hamiltonian, nev=nev, tol=tol, dtype=out_dtype, start=start, precision=precision)
    log.info("Obtained eigenvalues %s in %.3f s (%d Lanczos steps)", list(res.eigenvalues),
             time.perf_counter() - t0, res.iterations)
    vecs = np.asarray(res.eigenvectors).T.copy()  # (nev, D): row c is eigenvector c
    if cfg.datatype == "float32":
        vecs = vecs.astype(np.float32 if is_real else np.complex64)
    g = root.require(HAMILTONIAN_PATH)
    _overwrite(g, "eigenvalues", np.asarray(res.eigenvalues, dtype=np.float64), HAMILTONIAN_PATH)
    _overwrite(g, "eigenvectors", vecs, HAMILTONIAN_PATH)
    _overwrite(g, "residuals", np.asarray(res.residuals, dtype=np.float64), HAMILTONIAN_PATH)
    _save(cfg.output, root)
    return res


def compute_expectations(env: Environment, root: hdf5.Group, eigenvectors: np.ndarray) -> None:
    g = root.require(OBSERVABLES_PATH)
    X = np.asfortranarray(eigenvectors)
    for name, op in env.observables:
        log.info("Computing expectation values of %s...", name)
        m = I.expectation(op, X)
        log.info("Obtained expectation values %s", list(m))
        _overwrite(g, name, m.astype(np.complex128), OBSERVABLES_PATH)
    if env.observables:
        _save(env.config.output, root)


def run(config, debug: bool = False, warm_start: bool = True, precision: int = L.SED_PRECISION_FP64):
    """runApp: the whole YAML-to-HDF5 flow. `config` is a path or a ConfigSpec.
    Returns the EighResult of the Hamiltonian."""
    if debug:
        L.load().ls_enable_logging()
    cfg = read_config(config) if isinstance(config, str) else config
    env = to_environment(cfg)
    root = prepare_output_file(env)
    build_representatives(env, root)
    res = diagonalize(env, root, warm_start=warm_start, precision=precision)
    compute_expectations(env, root, res.eigenvectors)
    return res
