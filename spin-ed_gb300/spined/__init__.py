"""spined — host side of the GB300 exact-diagonalisation engine.

Mirrors SpinED's Haskell layers above the FFI:
  internal  — src/SpinED/Internal.hs (the ls_* / sed_* C ABI via ctypes)
  lattices  — the site/bond tables of SpinED's example configurations
  model     — building a basis and Hamiltonian from a lattice description
"""
from . import internal, lattices  # noqa: F401
from .model import build_model  # noqa: F401
