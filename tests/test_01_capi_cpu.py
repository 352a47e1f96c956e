"""libsed's C ABI on the CPU: the library loads, exports every symbol that
include/sed.h declares, validates input like the reference
(src/SpinED/Internal.hs:109-112,211-224; test/Spec.hs) and its symmetry plan
(Benes networks + shift subgroup) canonicalises exactly like the oracle.
No compute kernel runs here."""
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    txt = open(os.path.join(ROOT, "include", "sed.h")).read()
    return sorted(set(re.findall(r"^SED_API [^(]*?\b((?:ls|sed)_\w+)\(", txt, re.M)))


def test_exports_every_declared_symbol(sed):
    import subprocess
    from spined import _lib
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (\w+)", out))
    decl = declared_symbols()
    assert len(decl) >= 40
    missing = [s for s in decl if s not in exported]
    assert not missing, missing
    # ctypes signatures cover the same set
    assert sorted(n for n, _, _ in _lib.SIGNATURES) == decl


def test_spec_symmetries(sed, pins):
    p = pins["spec_periodicity"]["value"]
    s = sed.mk_symmetry(p["permutation"], p["sector"])
    assert sed.get_sector(s) == 0 and sed.get_periodicity(s) == 2 and sed.get_phase(s) == 0.0
    for key, code in (("spec_invalid_permutation", 6), ("spec_invalid_sector", 7)):
        v = pins[key]["value"]
        with pytest.raises(sed.LatticeSymmetriesException) as e:
            sed.mk_symmetry(v["permutation"], v["sector"])
        assert e.value.code == code
    with pytest.raises(sed.SpinEDException):
        sed.mk_symmetry([0, -1], 0)
    with pytest.raises(sed.SpinEDException):
        sed.mk_symmetry([1, 0], -1)


def test_spec_groups(sed, pins):
    v = pins["spec_group_size"]["value"]
    g = sed.mk_group([sed.mk_symmetry(p, s) for p, s in v["generators"]])
    assert sed.get_group_size(g) == v["size_permutations"]
    bad = pins["spec_incompatible_sectors"]["value"]
    with pytest.raises(sed.LatticeSymmetriesException) as e:
        sed.mk_group([sed.mk_symmetry(p, s) for p, s in bad["generators"]])
    assert e.value.code == 11
    assert sed.get_group_size(sed.mk_group([])) == 1


def test_spec_basis_validation(sed, pins):
    g = sed.mk_group([])
    with pytest.raises(sed.SpinEDException):
        sed.mk_basis(g, pins["spec_negative_spins"]["value"]["number_spins"])
    with pytest.raises(sed.SpinEDException):
        sed.mk_basis(g, 4, hamming_weight=-1)
    with pytest.raises(sed.SpinEDException):
        sed.mk_basis(g, 4, spin_inversion=2)
    with pytest.raises(sed.LatticeSymmetriesException):
        sed.mk_basis(g, 65)
    with pytest.raises(sed.LatticeSymmetriesException):
        sed.mk_basis(g, 5, hamming_weight=2, spin_inversion=1)  # inversion needs n/2
    g4 = sed.mk_group([sed.mk_symmetry([1, 2, 3, 0], 0)])
    with pytest.raises(sed.LatticeSymmetriesException):
        sed.mk_basis(g4, 6)  # group acts on 4 sites
    b = sed.mk_basis(g4, 4, 2)
    with pytest.raises(sed.LatticeSymmetriesException) as e:
        sed.get_number_states(b)
    assert e.value.code == 14  # not built


def test_spec_interactions(sed, pins):
    v = pins["spec_real_interaction"]["value"]
    x = sed.mk_interaction(v["matrix"], v["sites"])
    assert sed.is_real_interaction(x) is True
    y = sed.mk_interaction([[0, [0, -1]], [[0, 1], 0]], [[0]])
    assert sed.is_real_interaction(y) is False
    with pytest.raises(sed.SpinEDException):
        sed.mk_interaction([[1, 2], [3, 4]], [])
    with pytest.raises(sed.SpinEDException):
        sed.mk_interaction([[1, 2, 1], [4, 2, 1], [1, -2, 3]], [[0, 0, 0], [1, 1, 1]])  # 3x3 for 3 sites
    with pytest.raises(sed.SpinEDException):
        sed.mk_interaction([[1, 0], [0, 1]], [[0], [1, 2]])
    with pytest.raises(sed.LatticeSymmetriesException):
        sed.mk_interaction(np.eye(4).tolist(), [[1, 1]])  # repeated site
    g = sed.mk_group([])
    b = sed.mk_basis(g, 4)
    with pytest.raises(sed.LatticeSymmetriesException):
        sed.mk_operator(b, [sed.mk_interaction(np.eye(4).tolist(), [[0, 7]])])  # site beyond n


def test_error_strings(sed):
    from spined import _lib
    msg = _lib.error_message(6)
    assert "permutation" in msg
    assert _lib.error_message(0) == "success"


def random_states(rng, n, hw, count):
    out = []
    for _ in range(count):
        if hw is None:
            out.append(int(rng.integers(0, 2**min(n, 62))) if n <= 62 else int(rng.integers(0, 2**62)) << 2)
        else:
            bits = rng.choice(n, hw, replace=False)
            out.append(int(sum(1 << int(b) for b in bits)))
    return out


CASES = [
    ("chain24", 24, 12, 1, "chain", [0, 0]),
    ("chain40", 40, 20, 1, "chain", [0, 0]),
    ("chain20_k10_pm", 20, 10, -1, "chain", [10, 1]),
    ("chain12_k5", 12, 6, None, "chain", [5]),
    ("square6", 36, 18, 1, "square6", [0] * 5),
    ("square4_inv-", 16, 8, -1, "square4", [0] * 5),
    ("ring10_nohw", 10, None, None, "chain", [3]),
]


@pytest.mark.parametrize("name,n,hw,inv,kind,secs", CASES, ids=[c[0] for c in CASES])
def test_plan_canonicalises_like_oracle(sed, oracle, name, n, hw, inv, kind, secs):
    from spined import lattices
    if kind == "chain":
        gens = [lattices.chain_translation(n), lattices.chain_parity(n)]
    else:
        gens = lattices.square_symmetries(int(kind[-1]))
    gens = list(zip(gens, secs))  # zip drops generators without a sector
    b = sed.mk_basis(sed.mk_group([sed.mk_symmetry(p, s) for p, s in gens]), n, hw, inv)
    ob = oracle.Basis(n, hw, inv, gens)
    Lo = ob.group.L * (2 if (inv == -1 and ob.group.L % 2) else 1)
    rng = np.random.default_rng(7)
    for x in random_states(rng, n, hw, 1500):
        r, ph, L = b.state_info(x)
        r2, ph2, _ = ob.state_info(x)
        assert r == r2, (x, r, r2)
        if ob.representative_weight(r2):
            assert ph * Lo == ph2 * L


def _shear(L):
    """(x, y) -> (x, y + x): maps the rows of an L x L torus onto diagonals."""
    idx = lambda x, y: (y % L) * L + (x % L)
    return [idx(x, y + x) for y in range(L) for x in range(L)]


LINE_CASES = [
    # name, n, hw, inv, generators (permutation, sector), line tables, columns
    ("square4_full", 16, 8, 1, lambda lt: [(g, 0) for g in lt.square_symmetries(4)], 1, 1),
    ("square6_inv-", 36, 18, -1, lambda lt: [(g, 0) for g in lt.square_symmetries(6)], 1, 1),
    ("square6_C4_only", 36, 18, 1, lambda lt: [(g, 0) for g in lt.square_symmetries(6)[:2] + lt.square_symmetries(6)[4:]], 1, 1),
    ("square4_momentum", 16, 8, None, lambda lt: [(g, s) for g, s in zip(lt.square_symmetries(4)[:2], (1, 2))], 1, 0),
    ("rect6x4_reflections", 24, 12, 1, lambda lt: [(g, 0) for g in lt.rect_translations(6, 4)] + [
        ([(y * 6) + (5 - x) for y in range(4) for x in range(6)], 0),
        ([((3 - y) * 6) + x for y in range(4) for x in range(6)], 0)], 1, 0),
    ("square4_shear", 16, 8, None, lambda lt: [(g, 0) for g in lt.square_symmetries(4)[:2]] + [(_shear(4), 0)], 0, 0),
]


@pytest.mark.parametrize("name,n,hw,inv,gens,lines,cols", LINE_CASES, ids=[c[0] for c in LINE_CASES])
def test_line_table_plans(sed, capfd, name, n, hw, inv, gens, lines, cols):
    """Row-structured plans: the line tables are built exactly when every row
    of every coset image is a row or a column of the word; the plan builder
    checks the line-table test against the explicit group on random words
    and fails the basis creation on any mismatch."""
    from spined import _lib as L, lattices
    lib = L.load()
    lib.ls_enable_logging()
    try:
        g = sed.mk_group([sed.mk_symmetry(p, s) for p, s in gens(lattices)])
        sed.mk_basis(g, n, hw, inv)
    finally:
        lib.ls_disable_logging()
    err = capfd.readouterr().err
    assert "mode 1" in err, err  # every case is row-structured
    m = re.search(r"line tables: (\d) \(columns: (\d)\)", err)
    assert m, err
    assert (int(m.group(1)), int(m.group(2))) == (lines, cols), err


def _layout(lib, work, max_ctas, fixed, grid):
    import ctypes as C
    n = len(work)
    w = (C.c_double * n)(*work)
    m = (C.c_uint32 * n)(*max_ctas)
    group_of = (C.c_uint32 * n)()
    ncta = (C.c_uint32 * max(grid, 1))()
    nprob = (C.c_uint32 * max(grid, 1))()
    ng = lib.sed_debug_batched_layout(n, w, m, fixed, grid, group_of, ncta, nprob)
    return ng, list(group_of), list(ncta[:ng]), list(nprob[:ng])


def _makespan(work, fixed, group_of, ncta):
    t = [0.0] * len(ncta)
    for i, g in enumerate(group_of):
        t[g] += fixed + work[i] / ncta[g]
    return max(t)


@pytest.mark.parametrize("count,grid", [(128, 304), (128, 152), (128, 456), (1, 304), (400, 304), (1000, 152)])
def test_batched_layout(sed, count, grid):
    """The persistent batched launch's group layout (host logic of
    sed_eigh_batched): every problem lies in exactly one group, the groups use
    at most `grid` CTAs and no group more than its problems' slices, a group
    that solves several problems one after another has one CTA, and the
    modelled makespan is no worse than one group per problem with CTAs in
    proportion to work (the layout it replaced), on chain-like sizes."""
    from spined import _lib as L
    lib = L.load()
    rng = np.random.default_rng(count * 7 + grid)
    sizes = {16: 201, 18: 675, 20: 2309, 22: 8016, 24: 28968, 26: 100006, 28: 361270}
    D = [sizes[int(n)] for n in rng.choice(np.arange(16, 29, 2), size=count)]
    work = [float(d) * 100.0 for d in D]
    max_ctas = [(d + 31) // 32 for d in D]
    fixed = 1400.0 * 100.0
    ng, group_of, ncta, nprob = _layout(lib, work, max_ctas, fixed, grid)
    assert 1 <= ng <= grid
    assert sum(ncta) <= grid
    assert sorted(set(group_of)) == list(range(ng))
    assert [group_of.count(g) for g in range(ng)] == nprob
    for g in range(ng):
        assert ncta[g] >= 1
        if nprob[g] > 1:
            assert ncta[g] == 1
        else:
            (i,) = [k for k in range(count) if group_of[k] == g]
            assert ncta[g] <= max_ctas[i]
    new = _makespan(work, fixed, group_of, ncta)
    if count <= grid:  # the proportional layout: one CTA each, the rest by work
        extra = grid - count
        tot = sum(work)
        n = [1 + int(w / tot * extra) for w in work]
        rem = sorted(range(count), key=lambda i: -(w / tot * extra - int(w / tot * extra)) if (w := work[i]) else 0)
        for i in rem[: grid - sum(n)]:
            n[i] += 1
        n = [max(1, min(k, m)) for k, m in zip(n, max_ctas)]
        old = max(fixed + w / k for w, k in zip(work, n))
        assert new <= old * (1 + 1e-9), (new, old)
    # within 1.5x of a bound no layout beats: the largest problem on all the
    # CTAs it may use, or all the work spread evenly over the grid
    bound = max(max(fixed + w / min(m, grid) for w, m in zip(work, max_ctas)),
                sum(w + fixed for w in work) / grid)
    assert bound * (1 - 1e-9) <= new <= 1.5 * bound, (new, bound)


def test_batched_layout_edges(sed):
    from spined import _lib as L
    lib = L.load()
    ng, group_of, ncta, nprob = _layout(lib, [5e6], [1000], 1e3, 304)
    assert (ng, group_of, ncta, nprob) == (1, [0], [304], [1])
    ng, group_of, ncta, nprob = _layout(lib, [5e6], [7], 1e3, 304)  # capped by its slices
    assert (ng, ncta) == (1, [7])
    ng, group_of, ncta, nprob = _layout(lib, [0.0] * 10, [1] * 10, 0.0, 4)
    assert 1 <= ng <= 4 and sum(nprob) == 10 and all(c == 1 for c in ncta)
    assert _layout(lib, [1.0, -1.0], [1, 1], 0.0, 4)[0] == 0
    assert _layout(lib, [1.0], [1], 0.0, 0)[0] == 0
