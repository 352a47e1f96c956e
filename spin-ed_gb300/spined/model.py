"""Basis + Hamiltonian from a lattice description, the toBasis/toOperator
steps of src/SpinED.hs:175-200 (symmetries -> group -> basis; terms ->
interactions -> operator)."""
from __future__ import annotations

from dataclasses import dataclass

from . import internal as I
from .lattices import Model


@dataclass
class Built:
    model: Model
    group: I.SymmetryGroup
    basis: I.SpinBasis
    hamiltonian: I.Operator
    interactions: list


def build_model(m: Model, build: bool = True) -> Built:
    """toBasis + toOperator (src/SpinED.hs:178-200); builds the basis if asked."""
    if m.number_spins > 64:
        raise I.SpinEDException(
            f"invalid number_spins: {m.number_spins}; exact diagonalization is not feasible "
            "for systems larger than 64 spins")
    syms = [I.mk_symmetry(p, s) for p, s in m.symmetries]
    group = I.mk_group(syms)
    basis = I.mk_basis(group, m.number_spins, m.hamming_weight, m.spin_inversion)
    terms = [I.mk_interaction(mat, sites) for mat, sites in m.terms]
    op = I.mk_operator(basis, terms)
    if build:
        I.build_basis(basis)
    return Built(m, group, basis, op, terms)
