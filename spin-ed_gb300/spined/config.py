"""SpinED's configuration (src/SpinED.hs:81-173) read from YAML.

Field names, defaults and errors follow the reference's FromJSON instances:
``basis`` (number_spins, hamming_weight?, spin_inversion?, symmetries of
{permutation, sector}), ``hamiltonian`` and each of ``observables`` as
{name, terms of {matrix, sites}} with complex entries written as numbers or
[re, im] pairs, and the optional output (default
"exact_diagonalization_result.h5"), number_vectors (1), precision (0.0),
datatype ("float64"; "float32" accepted), max_primme_basis_size,
max_primme_block_size and min_primme_restart_size.
"""
from __future__ import annotations

from dataclasses import dataclass, field

from . import yaml_subset


class ConfigError(ValueError):
    """A configuration the reference's parser would reject."""


@dataclass
class SymmetrySpec:  # SpinED.hs:81-88
    permutation: list
    sector: int


@dataclass
class BasisSpec:  # SpinED.hs:94-102
    number_spins: int
    hamming_weight: int | None
    spin_inversion: int | None
    symmetries: list


@dataclass
class InteractionSpec:  # SpinED.hs:122-129
    matrix: list  # rows of complex
    sites: list


@dataclass
class OperatorSpec:  # SpinED.hs:131-138
    name: str
    terms: list


@dataclass
class ConfigSpec:  # SpinED.hs:157-173
    basis: BasisSpec
    hamiltonian: OperatorSpec
    observables: list
    output: str = "exact_diagonalization_result.h5"
    number_vectors: int = 1
    precision: float = 0.0
    datatype: str = "float64"
    max_primme_basis_size: int = 0
    max_primme_block_size: int = 1
    min_primme_restart_size: int = 0
    extra: dict = field(default_factory=dict)


def _req(obj: dict, key: str, what: str):
    if not isinstance(obj, dict):
        raise ConfigError(f"parsing {what} failed, expected Object")
    if key not in obj:
        raise ConfigError(f"parsing {what} failed, key \"{key}\" not found")
    return obj[key]


def _int(v, what: str) -> int:
    if isinstance(v, bool) or not isinstance(v, (int, float)) or (isinstance(v, float) and not v.is_integer()):
        raise ConfigError(f"parsing {what} failed, expected an integer, but got {v!r}")
    return int(v)


def _complex(v, what: str) -> complex:  # SpinED.hs:112-120
    if isinstance(v, bool):
        raise ConfigError(f"parsing Complex failed in {what}: {v!r}")
    if isinstance(v, (int, float)):
        return complex(float(v), 0.0)
    if isinstance(v, list) and len(v) == 2 and all(isinstance(x, (int, float)) and not isinstance(x, bool) for x in v):
        return complex(float(v[0]), float(v[1]))
    raise ConfigError(f"parsing Complex failed in {what}: expected a number or [re, im], got {v!r}")


def parse_symmetry(v) -> SymmetrySpec:
    perm = _req(v, "permutation", "symmetry")
    if not isinstance(perm, list):
        raise ConfigError("parsing symmetry failed, permutation must be a list")
    return SymmetrySpec([_int(p, "permutation") for p in perm], _int(_req(v, "sector", "symmetry"), "sector"))


def parse_basis(v) -> BasisSpec:
    syms = _req(v, "symmetries", "basis")
    if not isinstance(syms, list):
        raise ConfigError("parsing basis failed, symmetries must be a list")
    hw = v.get("hamming_weight")
    inv = v.get("spin_inversion")
    return BasisSpec(_int(_req(v, "number_spins", "basis"), "number_spins"),
                     None if hw is None else _int(hw, "hamming_weight"),
                     None if inv is None else _int(inv, "spin_inversion"),
                     [parse_symmetry(s) for s in syms])


def parse_interaction(v) -> InteractionSpec:
    m = _req(v, "matrix", "interaction")
    s = _req(v, "sites", "interaction")
    if not isinstance(m, list) or not all(isinstance(r, list) for r in m):
        raise ConfigError("parsing interaction failed, matrix must be a list of rows")
    if not isinstance(s, list) or not all(isinstance(t, list) for t in s):
        raise ConfigError("parsing interaction failed, sites must be a list of lists")
    return InteractionSpec([[_complex(x, "matrix") for x in row] for row in m],
                           [[_int(i, "sites") for i in t] for t in s])


def parse_operator(v) -> OperatorSpec:
    name = _req(v, "name", "operator")
    terms = _req(v, "terms", "operator")
    if not isinstance(terms, list):
        raise ConfigError("parsing operator failed, terms must be a list")
    return OperatorSpec(str(name), [parse_interaction(t) for t in terms])


def parse_config(v) -> ConfigSpec:
    if not isinstance(v, dict):
        raise ConfigError("parsing config failed, expected Object")
    obs = _req(v, "observables", "config")
    if not isinstance(obs, list):
        raise ConfigError("parsing config failed, observables must be a list")
    dt = v.get("datatype", "float64")
    if dt is None:
        dt = "float64"
    if not isinstance(dt, str) or dt.lower() not in ("float32", "float64"):  # SpinED.hs:146-155
        raise ConfigError(f"parsing Datatype failed, expected either 'float32' or 'float64', but got '{dt}'")
    known = {"basis", "hamiltonian", "observables", "output", "number_vectors", "precision", "datatype",
             "max_primme_basis_size", "max_primme_block_size", "min_primme_restart_size"}

    def opt(key, default, conv):
        x = v.get(key)
        return default if x is None else conv(x)

    return ConfigSpec(
        basis=parse_basis(_req(v, "basis", "config")),
        hamiltonian=parse_operator(_req(v, "hamiltonian", "config")),
        observables=[parse_operator(o) for o in obs],
        output=opt("output", "exact_diagonalization_result.h5", str),
        number_vectors=opt("number_vectors", 1, lambda x: _int(x, "number_vectors")),
        precision=opt("precision", 0.0, float),
        datatype=dt.lower(),
        max_primme_basis_size=opt("max_primme_basis_size", 0, lambda x: _int(x, "max_primme_basis_size")),
        max_primme_block_size=opt("max_primme_block_size", 1, lambda x: _int(x, "max_primme_block_size")),
        min_primme_restart_size=opt("min_primme_restart_size", 0, lambda x: _int(x, "min_primme_restart_size")),
        extra={k: x for k, x in v.items() if k not in known},
    )


def read_config(path: str) -> ConfigSpec:
    """readConfig (SpinED.hs:252-261)."""
    try:
        return parse_config(yaml_subset.load(path))
    except yaml_subset.YamlError as e:
        raise ConfigError(f"{path}: {e}") from None


def loads_config(text: str) -> ConfigSpec:
    return parse_config(yaml_subset.loads(text))
