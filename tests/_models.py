"""Test helpers: one lattice Model -> (libsed objects, oracle objects)."""
import numpy as np


def oracle_terms(oracle, model):
    return [oracle.Term(np.array(m, dtype=complex), np.array(s)) for m, s in model.terms]


def both(sed, oracle, model, build=True):
    from spined.model import build_model
    built = build_model(model, build=build)
    ob = oracle.Basis(model.number_spins, model.hamming_weight, model.spin_inversion, model.symmetries)
    ob.build()
    oop = oracle.Operator(ob, oracle_terms(oracle, model))
    return built, ob, oop


def random_complex_term(rng, k, hermitian=True):
    d = 2**k
    a = rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d))
    return (a + a.conj().T) / 2 if hermitian else a
