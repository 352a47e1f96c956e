"""The learned start vector (sed_mlp_*): forward pass, loss and gradients of
the GPU kernels against the FP64 CPU oracle (oracle/mlp_oracle.py), the
|psi|^2 sampler against the vector it samples, and what a trained network
gains over the random start of the plain method."""
import numpy as np
import pytest

import mlp_oracle as M
from spined import lattices
from spined.model import build_model

pytestmark = pytest.mark.gpu


def _net(n, h, mask=0, seed=3):
    from spined.learned import Mlp
    return Mlp(n, h, sign_mask=mask, seed=seed)


def _random_states(rng, n, N):
    return rng.integers(0, 2 ** min(n, 63), size=N, dtype=np.uint64)


@pytest.mark.parametrize("n,h", [(20, 64), (36, 512)])
def test_forward_matches_oracle(n, h):
    from spined import _lib as L
    rng = np.random.default_rng(n)
    net = _net(n, h)
    net.set_path(L.SED_MLP_PATH_SIMT)  # the CUDA-core path training uses
    p = net.get_params()
    p[h * n:h * n + h] = rng.normal(scale=0.1, size=h)  # nonzero biases
    net.set_params(p)
    st = _random_states(rng, n, 3000)
    got = net.forward(st)
    _, _, _, want = M.forward(p, n, h, st)
    # FP32 accumulation of up to 512 BF16 x FP32 products against FP64
    np.testing.assert_allclose(got, want, rtol=0, atol=2e-5 * max(1.0, np.abs(want).max()))


@pytest.mark.parametrize("n,h,count", [(36, 512, 3000), (20, 256, 129), (64, 128, 77), (24, 512, 1 << 15),
                                       (36, 512, 150001), (20, 256, 40000), (64, 128, 60001)])
def test_tensor_core_forward_matches_oracle(n, h, count):
    """The fused tcgen05 inference kernel against the FP64 oracle with h1
    rounded to BF16 as the kernel stores it; ragged last tiles included.
    The larger counts give every CTA of the persistent grid several tiles.
    Tolerance: the hardware tanh (relative error about 2^-11) and FP32
    accumulation in tensor memory, 4e-3 of the output scale."""
    rng = np.random.default_rng(count)
    net = _net(n, h, seed=count)
    assert net.uses_tensor_cores
    p = net.get_params()
    p[h * n:h * n + h] = rng.normal(scale=0.1, size=h)  # nonzero biases
    p[h * n + h + h * h:h * n + 2 * h + h * h] = rng.normal(scale=0.1, size=h)
    net.set_params(p)
    st = _random_states(rng, n, count)
    got = net.forward(st)
    _, _, _, want = M.forward(p, n, h, st, act_bf16=True)
    scale = max(1.0, np.abs(want).max())
    np.testing.assert_allclose(got, want, rtol=0, atol=4e-3 * scale)
    # and against the CUDA-core path (FP32 activations) to the same bound
    from spined import _lib as L
    net.set_path(L.SED_MLP_PATH_SIMT)
    assert not net.uses_tensor_cores
    np.testing.assert_allclose(got, net.forward(st), rtol=0, atol=4e-3 * scale)
    assert net.forward(st[:0]).shape == (0, 2)


def test_tensor_core_start_vector_matches_simt():
    """sed_mlp_start_vector over a built basis: the tensor-core inference and
    the CUDA-core path give the same vector up to the activation rounding."""
    from spined import _lib as L
    from spined.learned import Mlp
    b = build_model(lattices.heisenberg_chain(20))
    net = Mlp(20, 256, sign_mask=lattices.chain_sublattice_mask(20), seed=8)
    p = net.get_params()
    net.set_params(0.5 * p)  # small outputs: exp(a) stays well conditioned
    v_tc = net.start_vector(b.basis)
    net.set_path(L.SED_MLP_PATH_SIMT)
    v_simt = net.start_vector(b.basis)
    # signs come from the sign logit: they may differ only where it is ~0
    assert np.mean(np.sign(v_tc) != np.sign(v_simt)) < 1e-3
    np.testing.assert_allclose(np.abs(v_tc), np.abs(v_simt), rtol=2e-2, atol=1e-3 * np.abs(v_simt).max())


@pytest.mark.parametrize("n,h,mask,tc,N", [
    (16, 64, 0, False, 1500), (36, 512, lattices.square_sublattice_mask(6), False, 1500),
    (36, 512, lattices.square_sublattice_mask(6), True, 1500), (20, 128, 0, True, 1500),
    (64, 256, 0b1011, True, 1500), (7, 128, 0b101, True, 77), (36, 512, 0, True, 4096)])
def test_gradients_match_oracle(n, h, mask, tc, N):
    """Loss and gradient of one batch. CUDA cores (FP32 activations) against
    the FP64 oracle; tensor cores (the tcgen05 training step, BF16
    activations, weight gradients through transposed operand reads, ragged
    last row tiles) against the oracle with the same BF16 rounding points."""
    from spined import _lib as L
    from spined.learned import Samples
    rng = np.random.default_rng(7 + N + h)
    net = _net(n, h, mask)
    if not tc:
        net.set_path(L.SED_MLP_PATH_SIMT)
    assert net.uses_tensor_cores == tc
    p = net.get_params()
    p[h * n:h * n + h] = rng.normal(scale=0.1, size=h)  # nonzero biases
    net.set_params(p)
    s = Samples(_random_states(rng, n, N), rng.normal(size=N).astype(np.float32),
                rng.integers(0, 2, size=N).astype(np.float32))
    loss, g = net.loss_grad(s)
    want_loss, want_g = M.loss_grad(p, n, h, s.states, s.t_abs.astype(np.float64), s.t_sign, mask, act_bf16=tc)
    assert loss == pytest.approx(want_loss, rel=1e-5)
    # per-block tolerance: FP32 sums over N samples against FP64 (with BF16
    # activations also a rare rounding flip of one activation, 2^-8 of it)
    tol = 1e-3 if tc else 2e-4
    o = 0
    for name, k in [("W1", h * n), ("b1", h), ("W2", h * h), ("b2", h), ("W3", 2 * h), ("b3", 2)]:
        gg, ww = g[o:o + k], want_g[o:o + k]
        np.testing.assert_allclose(gg, ww, rtol=0, atol=tol * np.abs(ww).max() + 1e-9, err_msg=name)
        o += k
    if tc:  # the BF16 step is close to the FP32 one too
        _, g32 = M.loss_grad(p, n, h, s.states, s.t_abs.astype(np.float64), s.t_sign, mask)
        np.testing.assert_allclose(g, g32, rtol=0, atol=3e-2 * np.abs(g32).max())


@pytest.mark.parametrize("h,tc", [(64, False), (128, True)])
def test_training_lowers_the_loss(h, tc):
    from spined.learned import Samples
    rng = np.random.default_rng(11)
    n, N = 16, 1 << 14
    st = _random_states(rng, n, N)
    # a smooth target: log-amplitude = 0.1 * (number of up spins), sign = bit 0
    ones = np.array([bin(int(v)).count("1") for v in st], dtype=np.float32)
    s = Samples(st, 0.1 * ones, (st & np.uint64(1)).astype(np.float32))
    net = _net(n, h)
    assert net.uses_tensor_cores == tc
    l0, _ = net.loss_grad(s)
    l1 = net.train(s, epochs=20, batch=1000, lr=3e-3, seed=1)  # ragged: 16 batches of 1000, 384 samples unused
    l2, _ = net.loss_grad(s)
    assert l2 < 0.1 * l0, (l0, l1, l2)
    # a second network, same seed: both paths add every partial sum in a fixed order (no atomic adds), so the
    # trajectory is bit-identical
    net2 = _net(n, h)
    l1b = net2.train(s, epochs=20, batch=1000, lr=3e-3, seed=1)
    assert l1b == l1
    np.testing.assert_array_equal(net2.get_params(), net.get_params())


def test_sampler_labels_and_frequencies(sed):
    from spined.learned import sample
    b = build_model(lattices.heisenberg_chain(16))
    res = sed.eigh(b.hamiltonian)
    psi = res.eigenvectors[:, 0]
    reps = sed.basis_get_states(b.basis)
    norms = np.zeros(len(reps))
    import ctypes as C
    from spined import _lib as L
    assert L.load().sed_basis_get_norms(b.basis.ptr, C.c_void_p(norms.ctypes.data)) == 0
    n = 1 << 18
    s = sample(b.basis, psi, n, seed=9)
    idx = np.searchsorted(reps, s.states)
    assert np.all(reps[idx] == s.states)
    np.testing.assert_allclose(s.t_abs, np.log(np.abs(psi[idx]) * norms[idx]), rtol=0, atol=1e-5)
    sigma = 1.0 if np.sum(psi * np.abs(psi)) >= 0 else -1.0  # global sign fixed (sign_mask 0)
    np.testing.assert_array_equal(s.t_sign, (sigma * psi[idx] > 0).astype(np.float32))
    # -psi is the same eigenvector: same samples, same labels
    s_neg = sample(b.basis, -psi, 1000, seed=9)
    np.testing.assert_array_equal(s_neg.t_sign, s.t_sign[:1000])
    # with a sublattice sign prior the sign is fixed against the prior
    mask = lattices.chain_sublattice_mask(16)
    prior = np.array([(-1) ** bin(int(r) & mask).count("1") for r in reps])
    sig_m = 1.0 if np.sum(prior * psi * np.abs(psi)) >= 0 else -1.0
    s_m = sample(b.basis, -psi, 1000, seed=9, sign_mask=mask)
    np.testing.assert_array_equal(s_m.t_sign, (sig_m * psi[idx[:1000]] > 0).astype(np.float32))
    # frequencies against psi^2: every representative within 5 sigma
    p = psi ** 2 / np.sum(psi ** 2)
    counts = np.bincount(idx, minlength=len(reps))
    sigma = np.sqrt(n * p * (1 - p)) + 1
    assert np.all(np.abs(counts - n * p) <= 5 * sigma)
    # the same seed gives the same samples
    s2 = sample(b.basis, psi, 1000, seed=9)
    np.testing.assert_array_equal(s2.states, s.states[:1000])


def test_learned_start_beats_random_start(sed):
    """J1-J2 ring of 24 spins: ground states at J2 = 0, 0.1, 0.2 train the
    network; at J2 = 0.3 its start vector must need fewer Lanczos steps than
    the plain method's random start, and both must reach the same eigenpair."""
    from spined.learned import Mlp, Samples, sample
    n = 24
    parts = []
    for k, j2 in enumerate([0.0, 0.1, 0.2]):
        b = build_model(lattices.heisenberg_chain(n, j2=j2))
        r = sed.eigh(b.hamiltonian)
        parts.append(sample(b.basis, r.eigenvectors[:, 0], 1 << 16, seed=k,
                            sign_mask=lattices.chain_sublattice_mask(n)))
    data = Samples.concat(parts)
    net = Mlp(n, 128, sign_mask=lattices.chain_sublattice_mask(n), seed=5)
    net.train(data, epochs=30, batch=2048, lr=2e-3, seed=2)
    target = build_model(lattices.heisenberg_chain(n, j2=0.3))
    v = net.start_vector(target.basis)
    rand = sed.eigh(target.hamiltonian, seed=1234)
    learned = sed.eigh(target.hamiltonian, start=v / np.linalg.norm(v))
    psi = rand.eigenvectors[:, 0]
    overlap = abs(np.dot(v, psi)) / np.linalg.norm(v)
    assert overlap > 0.9, overlap
    assert learned.eigenvalues[0] == pytest.approx(rand.eigenvalues[0], rel=1e-10)
    assert learned.residuals[0] <= 1e-8
    assert learned.iterations < rand.iterations, (learned.iterations, rand.iterations)


# ------------------------------------------------------------ patch network
def _patch_net(L, h, mask=0, seed=3):
    from spined.learned import PatchMlp
    return PatchMlp(lattices.square_patches(L), h, sign_mask=mask, seed=seed)


def _patch_states(rng, L, N):
    n = L * L
    return rng.integers(0, 2 ** min(n, 63), size=N, dtype=np.uint64)


@pytest.mark.parametrize("L,h,count", [(4, 64, 1000), (6, 128, 777), (6, 256, 4099), (4, 128, 5)])
def test_patch_forward_matches_oracle(L, h, count):
    """Patch network inference against the oracle with BF16 activations:
    hidden 128 and 256 in the fused tensor-core kernel (site rows gathered
    from the patch table, outputs added per sample; hardware tanh, h2 kept in
    FP32: 4e-3 of the output scale), hidden 64 through the training step's
    forward GEMMs (1e-3). The sum over sites makes it invariant under
    translations of the torus."""
    rng = np.random.default_rng(L * 100 + h)
    net = _patch_net(L, h, seed=count)
    assert net.uses_tensor_cores
    p = net.get_params()
    P = 9
    p[h * P:h * P + h] = rng.normal(scale=0.1, size=h)
    net.set_params(p)
    st = _patch_states(rng, L, count)
    got = net.forward(st)
    want = M.patch_forward(p, h, st, lattices.square_patches(L), act_bf16=True)[3]
    scale = max(1.0, np.abs(want).max())
    np.testing.assert_allclose(got, want, rtol=0, atol=(4e-3 if h >= 128 else 1e-3) * scale)
    # translate every state by one site along x (site (x, y) -> (x + 1, y))
    perm = np.array([(y * L + (x + 1) % L) for y in range(L) for x in range(L)])
    bits = (st[:, None] >> np.arange(L * L, dtype=np.uint64)[None, :]) & np.uint64(1)
    moved = np.zeros_like(st)
    for i in range(L * L):
        moved |= bits[:, i] << np.uint64(perm[i])
    np.testing.assert_allclose(net.forward(moved), got, rtol=0, atol=1e-4 * scale)


@pytest.mark.parametrize("L,h,mask,N", [(4, 64, 0, 300), (6, 128, lattices.square_sublattice_mask(6), 77),
                                        (6, 64, 0, 1024)])
def test_patch_gradients_match_oracle(L, h, mask, N):
    from spined.learned import Samples
    rng = np.random.default_rng(L + h + N)
    net = _patch_net(L, h, mask)
    p = net.get_params()
    P = 9
    p[h * P:h * P + h] = rng.normal(scale=0.1, size=h)
    net.set_params(p)
    s = Samples(_patch_states(rng, L, N), rng.normal(size=N).astype(np.float32),
                rng.integers(0, 2, size=N).astype(np.float32))
    loss, g = net.loss_grad(s)
    want_loss, want_g = M.patch_loss_grad(p, h, s.states, lattices.square_patches(L), s.t_abs.astype(np.float64),
                                          s.t_sign, mask, act_bf16=True)
    assert loss == pytest.approx(want_loss, rel=1e-5)
    o = 0
    for name, k in [("W1", h * P), ("b1", h), ("W2", h * h), ("b2", h), ("W3", 2 * h), ("b3", 2)]:
        gg, ww = g[o:o + k], want_g[o:o + k]
        np.testing.assert_allclose(gg, ww, rtol=0, atol=1e-3 * np.abs(ww).max() + 1e-9, err_msg=name)
        o += k


def test_patch_network_transfers_between_lattices(sed):
    """Trained on the 4x4 ground state alone, the patch network is bound to
    the 6x6 torus: its outputs there match the oracle with the same
    parameters, and its start vector needs fewer Lanczos steps than the
    plain method's random start on the 6x6 ground state (D = 15.8 M)."""
    from spined import _lib as L
    from spined.learned import sample
    net = _patch_net(4, 64, mask=lattices.square_sublattice_mask(4), seed=5)
    with pytest.raises(Exception):
        net.set_path(L.SED_MLP_PATH_SIMT)  # patch networks run on the tensor cores only
    b4 = build_model(lattices.heisenberg_square(4))
    r4 = sed.eigh(b4.hamiltonian, tol=1e-10)
    data = sample(b4.basis, r4.eigenvectors[:, 0], 1 << 18, seed=3, sign_mask=lattices.square_sublattice_mask(4))
    net.train_decayed(data, epochs=32, batch=4096, lr=3e-3, seed=1)
    net.rebind(lattices.square_patches(6), lattices.square_sublattice_mask(6))
    b6 = build_model(lattices.heisenberg_square(6))
    reps = sed.basis_get_states(b6.basis)
    pick = reps[:: len(reps) // 1500][:1500]
    got = net.forward(pick)
    want = M.patch_forward(net.get_params(), 64, pick, lattices.square_patches(6), act_bf16=True)[3]
    np.testing.assert_allclose(got, want, rtol=0, atol=1e-3 * max(1.0, np.abs(want).max()))
    v = net.start_vector(b6.basis)
    rand = sed.eigh(b6.hamiltonian, seed=1234)
    learned = sed.eigh(b6.hamiltonian, start=v)
    psi = rand.eigenvectors[:, 0]
    overlap = abs(np.dot(v, psi)) / np.linalg.norm(v)
    assert overlap > 0.5, overlap
    assert learned.eigenvalues[0] == pytest.approx(rand.eigenvalues[0], rel=1e-10)
    assert learned.residuals[0] <= 1e-8
    assert learned.iterations < rand.iterations, (learned.iterations, rand.iterations)
