"""Generates tests/golden/reference_pins.json from the reference's own text.

The reference (twesterhout/spin-ed) pins only a handful of results: the
4-site Heisenberg ring of its README and the symmetry/group/basis checks of
test/Spec.hs. This script reads those files as text (it runs nothing from
the reference) and records each pin with the line it comes from, so the
tests can check the oracle and the library against them on machines where
the reference is not mounted.

Usage: python tests/golden/make_pins.py /path/to/reference
(or set SPINED_REFERENCE_DIR)
"""
from __future__ import annotations

import json
import os
import re
import sys


def line_of(lines: list[str], pattern: str) -> tuple[int, str]:
    for i, ln in enumerate(lines, 1):
        if re.search(pattern, ln):
            return i, ln
    raise SystemExit(f"pattern not found: {pattern}")


def main(ref: str) -> None:
    readme = open(os.path.join(ref, "README.md")).read().splitlines()
    spec = open(os.path.join(ref, "test", "Spec.hs")).read().splitlines()
    pins = []

    # README: representatives dataset has 16 entries; eigenvalue -8.
    n, ln = line_of(readme, r"DATASPACE\s+SIMPLE \{ \( 16 \) / \( 16 \) \}")
    pins.append({"id": "readme_ring4_dimension", "source": f"README.md:{n}", "value": 16,
                 "what": "4-site ring, no symmetries, no Hamming weight: 16 representatives"})
    n, ln = line_of(readme, r"\(0\):\s*-8")
    e0 = float(re.search(r"\(0\):\s*(-?\d+(\.\d+)?)", ln).group(1))
    pins.append({"id": "readme_ring4_e0", "source": f"README.md:{n}", "value": e0,
                 "what": "ground-state energy of the 4-site Heisenberg ring"})
    # The ring's sites and matrix (README.md usage block).
    n, ln = line_of(readme, r"sites: \[\[0, 1\], \[1, 2\], \[2, 3\], \[3, 0\]\]")
    pins.append({"id": "readme_ring4_sites", "source": f"README.md:{n}",
                 "value": [[0, 1], [1, 2], [2, 3], [3, 0]], "what": "bonds of the README example"})

    # test/Spec.hs
    n, ln = line_of(spec, r"getPeriodicity s₁ `shouldBe` 2")
    pins.append({"id": "spec_periodicity", "source": f"test/Spec.hs:{n}",
                 "value": {"permutation": [3, 2, 1, 0], "sector": 0, "periodicity": 2}})
    n, ln = line_of(spec, r"toSymmetry \(SymmetrySpec \[4, 3, 4, 1\]")
    pins.append({"id": "spec_invalid_permutation", "source": f"test/Spec.hs:{n}",
                 "value": {"permutation": [4, 3, 4, 1], "sector": 0, "throws": True}})
    n, ln = line_of(spec, r"toSymmetry \(SymmetrySpec \[4, 3, 2, 1, 0\] False 3\)")
    pins.append({"id": "spec_invalid_sector", "source": f"test/Spec.hs:{n}",
                 "value": {"permutation": [4, 3, 2, 1, 0], "sector": 3, "throws": True}})
    n, ln = line_of(spec, r"getGroupSize g `shouldBe` 16")
    pins.append({"id": "spec_group_size", "source": f"test/Spec.hs:{n}",
                 "value": {"generators": [[[3, 2, 1, 0], 0], [[1, 2, 3, 0], 0]], "spin_inversion": True,
                           "size_with_inversion": 16, "size_permutations": 8},
                 "what": "D4 plus global spin flip (the flip is a basis field in the current API)"})
    n, ln = line_of(spec, r"mkGroup \[s₁, s₂', s₃\] `shouldThrow`")
    pins.append({"id": "spec_incompatible_sectors", "source": f"test/Spec.hs:{n}",
                 "value": {"generators": [[[3, 2, 1, 0], 0], [[1, 2, 3, 0], 1]], "throws": True}})
    n, ln = line_of(spec, r"BasisSpec \(-2\)")
    pins.append({"id": "spec_negative_spins", "source": f"test/Spec.hs:{n}",
                 "value": {"number_spins": -2, "throws": True}})
    n, ln = line_of(spec, r"sites = \[\[0\], \[2\]\]")
    pins.append({"id": "spec_real_interaction", "source": f"test/Spec.hs:{n}",
                 "value": {"matrix": [[1.0, 0.0], [0.0, -1.0]], "sites": [[0], [2]], "is_real": True}})

    # example/*.yaml: the lattice tables of the 6x6 and chain-40 workloads
    def ints(block):
        return [int(v) for v in re.findall(r"-?\d+", block)]

    sq = open(os.path.join(ref, "example", "heisenberg_square_6x6.yaml")).read()
    sq_lines = sq.splitlines()
    n, _ = line_of(sq_lines, r"permutation:")
    pairs = ints(re.search(r"sites:\s*\[(.*?)\]\]", sq, re.S).group(1) + "]")
    pins.append({"id": "example_square6_tables", "source": f"example/heisenberg_square_6x6.yaml:{n}",
                 "value": {"permutations": [ints(b) for b in re.findall(r"permutation:\s*\[([^\]]*)\]", sq)],
                           "bonds": [pairs[i:i + 2] for i in range(0, len(pairs), 2)]},
                 "what": "generators and nearest-neighbour bonds of the 6x6 periodic square lattice"})
    ch = open(os.path.join(ref, "example", "heisenberg_chain_40.yaml")).read()
    n, _ = line_of(ch.splitlines(), r"permutation:")
    perms = re.findall(r"permutation:\s*\[([^\]]*)\]", ch)
    pins.append({"id": "example_chain40_tables", "source": f"example/heisenberg_chain_40.yaml:{n}",
                 "value": {"translation": ints(perms[0]), "parity": ints(perms[1])},
                 "what": "translation and parity generators of the 40-site chain"})

    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_pins.json")
    with open(out, "w") as f:
        json.dump({"reference": "twesterhout/spin-ed", "generated_by": "tests/golden/make_pins.py",
                   "pins": pins}, f, indent=1)
    print(out)


if __name__ == "__main__":
    where = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("SPINED_REFERENCE_DIR")
    if not where:
        raise SystemExit("usage: make_pins.py REFERENCE_DIR (or set SPINED_REFERENCE_DIR)")
    main(where)
