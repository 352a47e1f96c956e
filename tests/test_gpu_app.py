"""The YAML-in / HDF5-out flow (app/Main.hs runApp) end to end on the GPU:
the README's 4-spin ring (E0 = -8, pinned from the reference's README), a
chain with observables and two vectors checked against the FP64 oracle, and
the resume contract: a second run loads /basis/representatives and starts
from the stored eigenvectors."""
import numpy as np
import pytest

from _models import both
from spined import app, hdf5
from spined import config as CF
from spined import lattices

pytestmark = pytest.mark.gpu


def _yaml_chain(n, out, nev=1, observables="[]", inv=1):
    perm = list(range(1, n)) + [0]
    bonds = [[i, (i + 1) % n] for i in range(n)]
    return f"""
basis:
  number_spins: {n}
  hamming_weight: {n // 2}
  spin_inversion: {inv}
  symmetries:
    - permutation: {perm}
      sector: 0
    - permutation: {list(reversed(range(n)))}
      sector: 0
hamiltonian:
  name: "Heisenberg Hamiltonian"
  terms:
    - matrix: [[1, 0, 0, 0], [0, -1, 2, 0], [0, 2, -1, 0], [0, 0, 0, 1]]
      sites: {bonds}
observables: {observables}
number_vectors: {nev}
output: "{out}"
"""


def test_readme_ring(tmp_path, pins):
    from test_03_frontend_cpu import README_CONFIG
    out = tmp_path / "readme.h5"
    cfg = CF.loads_config(README_CONFIG + f'output: "{out}"\n')
    res = app.run(cfg)
    assert res.eigenvalues[0] == pytest.approx(pins["readme_ring4_e0"]["value"], abs=1e-10)
    root = hdf5.read(str(out))
    assert sorted(root) == ["_workspace", "basis", "hamiltonian", "observables"]
    reps = root["basis"]["representatives"]
    assert reps.dtype == np.uint64 and reps.shape == (16,)
    h = root["hamiltonian"]
    assert h["eigenvalues"].shape == (1,) and h["eigenvectors"].shape == (1, 16) and h["residuals"].shape == (1,)
    assert h["eigenvalues"][0] == pytest.approx(-8.0, abs=1e-10)
    assert h["residuals"][0] <= 1e-8


def test_chain_with_observables(sed, oracle, tmp_path):
    n = 12
    out = tmp_path / "chain.h5"
    # total S^z^2-like observable: sum_i sigma^z_i sigma^z_{i+1} (diagonal), and the Hamiltonian itself
    zz = "[[1, 0, 0, 0], [0, -1, 0, 0], [0, 0, -1, 0], [0, 0, 0, 1]]"
    bonds = [[i, (i + 1) % n] for i in range(n)]
    obs = (f'\n  - name: "ZZ"\n    terms:\n      - matrix: {zz}\n        sites: {bonds}'
           f'\n  - name: "H"\n    terms:\n      - matrix: [[1, 0, 0, 0], [0, -1, 2, 0], [0, 2, -1, 0], [0, 0, 0, 1]]'
           f'\n        sites: {bonds}')
    cfg = CF.loads_config(_yaml_chain(n, out, nev=2, observables=obs))
    res = app.run(cfg)
    built, ob, oop = both(sed, oracle, lattices.heisenberg_chain(n))
    A = oop.sparse().real
    import scipy.sparse.linalg as sla
    want = np.sort(sla.eigsh(A, k=2, which="SA")[0])
    np.testing.assert_allclose(res.eigenvalues, want, rtol=1e-10)
    root = hdf5.read(str(out))
    np.testing.assert_array_equal(root["basis"]["representatives"], ob.reps)
    vecs = root["hamiltonian"]["eigenvectors"]
    assert vecs.shape == (2, len(ob.reps))
    e_h = root["observables"]["H"]
    assert e_h.dtype == np.complex128
    np.testing.assert_allclose(e_h.real, res.eigenvalues, rtol=1e-10)
    zz_want = [vecs[c] @ (oracle.Operator(ob, [oracle.Term(np.diag([1, -1, -1, 1]).astype(complex), np.array(bonds))]).sparse().real @ vecs[c]) for c in range(2)]
    np.testing.assert_allclose(root["observables"]["ZZ"].real, zz_want, rtol=1e-10)


def test_resume_loads_representatives_and_warm_starts(tmp_path):
    out = tmp_path / "resume.h5"
    cfg = CF.loads_config(_yaml_chain(16, out))
    first = app.run(cfg)
    reps = hdf5.read(str(out))["basis"]["representatives"].copy()
    second = app.run(cfg)  # /basis/representatives and /hamiltonian/eigenvectors exist now
    assert second.eigenvalues[0] == pytest.approx(first.eigenvalues[0], rel=1e-12)
    assert second.iterations < first.iterations
    np.testing.assert_array_equal(hdf5.read(str(out))["basis"]["representatives"], reps)


def test_float32_datatype(tmp_path):
    out = tmp_path / "f32.h5"
    cfg = CF.loads_config(_yaml_chain(12, out) + 'datatype: "float32"\n')
    app.run(cfg)
    v = hdf5.read(str(out))["hamiltonian"]["eigenvectors"]
    assert v.dtype == np.float32
