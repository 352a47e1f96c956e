"""Lattice builders for the workloads SpinED's examples describe.

The reference spells out site permutations and bond lists by hand in its
YAML examples (example/heisenberg_chain_40.yaml:9-31,
example/heisenberg_square_6x6.yaml:14-69); these functions generate the same
tables (row-major site numbering, site = y * L + x) so that configurations
of any size can be built programmatically.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

HEISENBERG = [[1, 0, 0, 0], [0, -1, 2, 0], [0, 2, -1, 0], [0, 0, 0, 1]]  # sigma . sigma


@dataclass
class Model:
    name: str
    number_spins: int
    hamming_weight: int | None
    spin_inversion: int | None
    symmetries: list[tuple[list[int], int]]
    terms: list[tuple[list[list[complex]], list[list[int]]]]  # (matrix, sites)
    meta: dict = field(default_factory=dict)


def chain_translation(n: int) -> list[int]:
    return [(i + 1) % n for i in range(n)]


def chain_parity(n: int) -> list[int]:
    return [n - 1 - i for i in range(n)]


def chain_bonds(n: int, distance: int = 1) -> list[list[int]]:
    return [[i, (i + distance) % n] for i in range(n)]


def heisenberg_chain(n: int, hamming_weight: int | None = None, momentum: int = 0, parity: int | None = 0,
                     spin_inversion: int | None = 1, j2: float = 0.0) -> Model:
    """Periodic chain with nearest (and optionally next-nearest, scaled j2) bonds.

    parity is the sector of the reflection (0 or 1) or None to leave it out.
    """
    hw = n // 2 if hamming_weight is None else hamming_weight
    syms = [(chain_translation(n), momentum)]
    if parity is not None:
        syms.append((chain_parity(n), parity))
    terms = [(HEISENBERG, chain_bonds(n, 1))]
    if j2:
        terms.append(([[j2 * v for v in row] for row in HEISENBERG], chain_bonds(n, 2)))
    inv = spin_inversion if (spin_inversion is not None and 2 * hw == n) else None
    return Model(f"chain{n}", n, hw, inv, syms, terms, {"j2": j2})


def square_symmetries(L: int) -> list[list[int]]:
    """Tx, Ty, reflection x -> L-1-x, reflection y -> L-1-y, rotation by 90 degrees."""
    idx = lambda x, y: (y % L) * L + (x % L)
    tx = [idx(x + 1, y) for y in range(L) for x in range(L)]
    ty = [idx(x, y + 1) for y in range(L) for x in range(L)]
    rx = [idx(L - 1 - x, y) for y in range(L) for x in range(L)]
    ry = [idx(x, L - 1 - y) for y in range(L) for x in range(L)]
    rot = [idx(L - 1 - y, x) for y in range(L) for x in range(L)]
    return [tx, ty, rx, ry, rot]


def rect_translations(Lx: int, Ly: int) -> list[list[int]]:
    """Tx, Ty on an Lx x Ly torus (site = y * Lx + x)."""
    idx = lambda x, y: (y % Ly) * Lx + (x % Lx)
    tx = [idx(x + 1, y) for y in range(Ly) for x in range(Lx)]
    ty = [idx(x, y + 1) for y in range(Ly) for x in range(Lx)]
    return [tx, ty]


def rect_bonds(Lx: int, Ly: int) -> list[list[int]]:
    """Nearest-neighbour bonds of an Lx x Ly torus."""
    idx = lambda x, y: (y % Ly) * Lx + (x % Lx)
    return [[idx(x, y), idx(x + 1, y)] for y in range(Ly) for x in range(Lx)] + \
           [[idx(x, y), idx(x, y + 1)] for y in range(Ly) for x in range(Lx)]


def square_bonds(L: int) -> list[list[int]]:
    """Nearest-neighbour bonds in the order of the reference's 6x6 example."""
    idx = lambda x, y: (y % L) * L + (x % L)
    out = []
    for y in range(L):
        for x in range(L):
            out.append([idx(x, y), idx(x + 1, y)])
            out.append([idx(x, y), idx(x, y + 1)])
    return out


def square_diagonals(L: int) -> list[list[int]]:
    idx = lambda x, y: (y % L) * L + (x % L)
    out = []
    for y in range(L):
        for x in range(L):
            out.append([idx(x, y), idx(x + 1, y + 1)])
            out.append([idx(x, y), idx(x - 1, y + 1)])
    return out


def heisenberg_square(L: int, spin_inversion: int | None = 1, j2: float = 0.0,
                      point_group: bool = True) -> Model:
    n = L * L
    gens = square_symmetries(L)
    if not point_group:
        gens = gens[:2]
    terms = [(HEISENBERG, square_bonds(L))]
    if j2:
        terms.append(([[j2 * v for v in row] for row in HEISENBERG], square_diagonals(L)))
    hw = n // 2
    inv = spin_inversion if 2 * hw == n else None
    return Model(f"square{L}x{L}", n, hw, inv, [(g, 0) for g in gens], terms, {"j2": j2})


def j1j2_chains(count: int = 128, seed: int = 2024) -> list[Model]:
    """The batched workload: N uniform over {16, 18, ..., 28}, J2/J1 uniform in [0, 0.6]."""
    rng = np.random.default_rng(seed)
    ns = rng.choice(np.arange(16, 29, 2), size=count)
    j2s = rng.uniform(0.0, 0.6, size=count)
    return [heisenberg_chain(int(n), j2=float(j)) for n, j in zip(ns, j2s)]


def square_sublattice_mask(L: int) -> int:
    """Bits of the sites with x + y even (one sublattice of the bipartite
    L x L torus, L even): the mask of the Marshall sign prior."""
    return sum(1 << ((y % L) * L + (x % L)) for y in range(L) for x in range(L) if (x + y) % 2 == 0)


def chain_sublattice_mask(n: int) -> int:
    """Even sites of a ring of even length n."""
    return sum(1 << i for i in range(0, n, 2))


def square_patches(L: int, radius: int = 1) -> np.ndarray:
    """(L*L, (2 radius + 1)^2) patch table of the L x L torus: row i lists the
    sites of the square window around site i, offsets (dx, dy) in row-major
    order, so every site's patch has the same shape on any L (the input of
    the size-independent patch network)."""
    idx = lambda x, y: (y % L) * L + (x % L)
    offs = [(dx, dy) for dy in range(-radius, radius + 1) for dx in range(-radius, radius + 1)]
    return np.array([[idx(x + dx, y + dy) for dx, dy in offs] for y in range(L) for x in range(L)], dtype=np.uint16)

