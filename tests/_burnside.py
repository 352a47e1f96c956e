"""Exact sector dimension by Burnside's lemma (an independent count).

The number of orbits of weight-w words whose stabiliser carries the trivial
character of a one-dimensional representation chi is
    D = (1/|G|) sum_g conj(chi(g)) |Fix_w(g)|.
For a permutation, fixed words are constant on cycles (a subset-sum over cycle
lengths); composed with spin inversion, bits alternate along every cycle, so
all cycles must be even and there are 2^(#cycles) fixed words.
"""
import numpy as np


def cycles(p):
    n, seen, out = len(p), [False] * len(p), []
    for i in range(n):
        if not seen[i]:
            L, j = 0, i
            while not seen[j]:
                seen[j] = True
                j = p[j]
                L += 1
            out.append(L)
    return out


def fixed_weight_count(cyc, w):
    poly = np.zeros(sum(cyc) + 1, dtype=object)
    poly[0] = 1
    for L in cyc:
        nxt = poly.copy()
        nxt[L:] = nxt[L:] + poly[: len(poly) - L]
        poly = nxt
    return int(poly[w]) if w is not None else int(sum(poly))


def sector_dimension(group, n, hw, inv):
    """group: oracle.Group (perms, phases mod L)."""
    total = 0j
    for p, ph in zip(group.perms, group.phases):
        chi = np.exp(2j * np.pi * int(ph) / group.L)  # conj of exp(-2 pi i ph / L)
        cyc = cycles(list(p))
        total += chi * fixed_weight_count(cyc, hw)
        if inv:
            fix = 2 ** len(cyc) if all(c % 2 == 0 for c in cyc) else 0
            total += chi * inv * fix
    order = len(group.perms) * (2 if inv else 1)
    d = total / order
    assert abs(d.imag) < 1e-6 and abs(d.real - round(d.real)) < 1e-6
    return int(round(d.real))
