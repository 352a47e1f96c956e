"""The start-vector MLP's CPU oracle (oracle/mlp_oracle.py), checked before it
is trusted: its analytic gradient against central finite differences, and
its BF16 rounding against torch's float32 -> bfloat16 conversion."""
import numpy as np
import pytest

import mlp_oracle as M


def _unpack64(q, n, h):
    out, o = {}, 0
    for name, shp in [("W1", (h, n)), ("b1", (h,)), ("W2", (h, h)), ("b2", (h,)), ("W3", (2, h)), ("b3", (2,))]:
        k = int(np.prod(shp))
        out[name] = q[o:o + k].reshape(shp)
        o += k
    return out


@pytest.mark.parametrize("mask", [0, 0b101101])
def test_gradient_matches_finite_differences(mask):
    rng = np.random.default_rng(5)
    n, h, N = 7, 6, 33
    size = h * n + h + h * h + h + 2 * h + 2
    p = (rng.integers(-96, 96, size=size) / 64).astype(np.float32)  # exactly representable in BF16
    st = rng.integers(0, 2 ** n, size=N).astype(np.uint64)
    ta = rng.normal(size=N)
    ts = rng.integers(0, 2, size=N).astype(np.float32)
    loss, g = M.loss_grad(p, n, h, st, ta, ts, mask)

    def f(q):
        w = _unpack64(q, n, h)
        x = M.spins(st, n)
        h1 = np.tanh(x @ w["W1"].T + w["b1"])
        h2 = np.tanh(h1 @ w["W2"].T + w["b2"])
        o = h2 @ w["W3"].T + w["b3"]
        y = np.abs(ts - M.parity(st, mask))
        a, s = o[:, 0], o[:, 1]
        return np.mean((a - ta) ** 2 + np.maximum(s, 0) - s * y + np.log1p(np.exp(-np.abs(s))))

    q = p.astype(np.float64)
    assert loss == pytest.approx(f(q), rel=1e-14)
    eps = 1e-6
    fd = np.array([(f(q + eps * e) - f(q - eps * e)) / (2 * eps) for e in np.eye(len(q))])
    np.testing.assert_allclose(g, fd, atol=1e-8, rtol=1e-6)


def test_bf16_rounding_matches_torch():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(1)
    x = np.concatenate([rng.normal(size=4000).astype(np.float32),
                        # ties: low 16 bits exactly 0x8000, both parities of bit 16
                        (np.arange(64, dtype=np.uint32) << 16 | 0x3F800000 | 0x8000).view(np.float32)])
    want = torch.from_numpy(x).to(torch.bfloat16).to(torch.float64).numpy()
    np.testing.assert_array_equal(M.bf16(x), want)


def test_spins_and_parity():
    st = np.array([0b0110, 0b1111, 0], dtype=np.uint64)
    np.testing.assert_array_equal(M.spins(st, 4)[0], [-1, 1, 1, -1])
    np.testing.assert_array_equal(M.parity(st, 0b0011), [1, 0, 0])


@pytest.mark.parametrize("mask", [0, 0b0110])
def test_patch_gradient_matches_finite_differences(mask):
    """The patch network (per-site MLP summed over sites): analytic gradient
    against central differences, and the same parameters on two lattice sizes."""
    rng = np.random.default_rng(9)
    h, P = 5, 3
    patches = np.array([[i, (i + 1) % 4, (i + 3) % 4] for i in range(4)])  # ring of 4, neighbours
    size = h * P + h + h * h + h + 2 * h + 2
    p = (rng.integers(-96, 96, size=size) / 64).astype(np.float32)
    st = rng.integers(0, 16, size=21).astype(np.uint64)
    ta = rng.normal(size=21)
    ts = rng.integers(0, 2, size=21).astype(np.float32)
    loss, g = M.patch_loss_grad(p, h, st, patches, ta, ts, mask)

    def f(q):
        w = _unpack64(q, P, h)
        x = M.patch_spins(st, patches)
        h1 = np.tanh(x @ w["W1"].T + w["b1"])
        h2 = np.tanh(h1 @ w["W2"].T + w["b2"])
        o = h2.sum(axis=1) @ w["W3"].T + w["b3"]
        y = np.abs(ts - M.parity(st, mask))
        a, s = o[:, 0], o[:, 1]
        return np.mean((a - ta) ** 2 + np.maximum(s, 0) - s * y + np.log1p(np.exp(-np.abs(s))))

    q = p.astype(np.float64)
    assert loss == pytest.approx(f(q), rel=1e-14)
    eps = 1e-6
    fd = np.array([(f(q + eps * e) - f(q - eps * e)) / (2 * eps) for e in np.eye(len(q))])
    np.testing.assert_allclose(g, fd, atol=1e-8, rtol=1e-6)
    # translation invariance: rotating every state of the ring leaves the outputs unchanged
    rot = ((st << np.uint64(1)) | (st >> np.uint64(3))) & np.uint64(15)
    np.testing.assert_allclose(M.patch_forward(p, h, rot, patches)[3], M.patch_forward(p, h, st, patches)[3],
                               rtol=1e-12)
