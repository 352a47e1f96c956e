"""ls_operator_matmat on the GPU against the oracle's pull-form matvec
(src/SpinED/Internal.hs:411-429), in all four dtypes, for host and device
buffers, strided blocks, both matvec forms, and ls_operator_expectation."""
import numpy as np
import pytest

from _models import both, random_complex_term
from spined import lattices
from spined import _lib as L

pytestmark = pytest.mark.gpu

# FP64 results differ from the oracle only by summation order.
RTOL64 = 1e-12
RTOL32 = 2e-5


def models():
    rng = np.random.default_rng(11)
    cx2 = random_complex_term(rng, 2)
    cx3 = random_complex_term(rng, 3)
    real3 = np.real(random_complex_term(rng, 3))
    return {
        "chain24": lattices.heisenberg_chain(24),
        "chain20_j2": lattices.heisenberg_chain(20, j2=0.35),
        "square4": lattices.heisenberg_square(4),
        "square4_j2": lattices.heisenberg_square(4, j2=0.5),
        "chain16_k5_complex": lattices.Model("c16k5", 16, 8, None, [(lattices.chain_translation(16), 5)],
                                             [(cx2.tolist(), lattices.chain_bonds(16))]),
        "chain12_3site": lattices.Model("c12t", 12, 6, 1, [(lattices.chain_translation(12), 0)],
                                        [(real3.tolist(), [[i, (i + 1) % 12, (i + 2) % 12] for i in range(12)])]),
        "chain10_3site_k2": lattices.Model("c10t", 10, None, None, [(lattices.chain_translation(10), 2)],
                                           [(cx3.tolist(), [[i, (i + 1) % 10, (i + 3) % 10] for i in range(10)])]),
        "field_1site_4site": lattices.Model("c8f", 8, None, None, [(lattices.chain_translation(8), 0)],
                                            [([[0.3, 1.0], [1.0, -0.3]], [[i] for i in range(8)]),
                                             (np.diag(np.arange(16) * 0.1).tolist(), [[i, (i + 1) % 8, (i + 2) % 8, (i + 3) % 8] for i in range(8)])]),
    }


MODELS = models()


@pytest.mark.parametrize("name", list(MODELS))
def test_matvec_matches_oracle(sed, oracle, name):
    built, ob, oop = both(sed, oracle, MODELS[name])
    D = len(ob.reps)
    rng = np.random.default_rng(3)
    x = rng.normal(size=D) + (0 if oop.is_real else 1j * rng.normal(size=D))
    want = oop.matvec(x)
    scale = np.abs(want).max()
    assert sed.is_operator_real(built.hamiltonian) == oop.is_real
    dts = [np.complex128, np.complex64] + ([np.float64, np.float32] if oop.is_real else [])
    for dt in dts:
        xv = x.astype(dt) if np.iscomplexobj(np.zeros(1, dt)) else x.real.astype(dt)
        y = sed.apply(built.hamiltonian, xv)
        ref = oop.matvec(xv.astype(np.complex128))
        tol = RTOL64 if dt in (np.float64, np.complex128) else RTOL32
        if not np.iscomplexobj(y):
            ref = ref.real
        np.testing.assert_allclose(y, ref, rtol=0, atol=tol * scale * 4)


def test_real_dtype_rejected_for_complex_operator(sed, oracle):
    built, ob, oop = both(sed, oracle, MODELS["chain16_k5_complex"])
    x = np.ones(len(ob.reps))
    with pytest.raises(sed.LatticeSymmetriesException) as e:
        sed.apply(built.hamiltonian, x)
    assert e.value.code == L.LS_OPERATOR_IS_COMPLEX


def test_dimension_mismatch(sed, oracle):
    built, ob, oop = both(sed, oracle, MODELS["chain24"])
    with pytest.raises(sed.LatticeSymmetriesException) as e:
        sed.apply(built.hamiltonian, np.ones(len(ob.reps) - 1))
    assert e.value.code == L.LS_DIMENSION_MISMATCH


def test_block_with_strides(sed, oracle):
    built, ob, oop = both(sed, oracle, MODELS["chain20_j2"])
    D = len(ob.reps)
    rng = np.random.default_rng(5)
    big = np.asfortranarray(rng.normal(size=(D + 7, 3)))
    x = big[:D, :]  # column stride D + 7
    yb = np.asfortranarray(np.zeros((D + 3, 3)))
    y = yb[:D, :]
    sed.inplace_apply(built.hamiltonian, x, y)
    for c in range(3):
        np.testing.assert_allclose(y[:, c], oop.matvec(x[:, c]).real, atol=1e-11)
    assert np.all(yb[D:, :] == 0)


def test_forms_agree_bit_for_bit(sed, oracle):
    """The on-the-fly and streamed forms sum the same elements in the same
    order, so they agree exactly."""
    import torch
    built, ob, oop = both(sed, oracle, MODELS["square4_j2"])
    D = len(ob.reps)
    x = torch.randn(D, dtype=torch.float64, device="cuda")
    y1 = torch.zeros_like(x)
    y2 = torch.zeros_like(x)
    lib = L.load()
    import ctypes as C
    torch.cuda.synchronize()
    from spined.internal import check_status
    op = built.hamiltonian
    check_status(lib.sed_operator_prepare(op.ptr, L.SED_FORM_ON_THE_FLY))
    assert op.stream_bytes == 0
    sed.inplace_apply(op, x, y1)  # on-the-fly form
    torch.cuda.synchronize()
    assert op.stream_bytes == 0
    op.prepare(L.SED_FORM_STREAM)
    assert op.stream_bytes > 0 and op.stream_elements > 0
    sed.inplace_apply(op, x, y2)  # streamed form
    torch.cuda.synchronize()
    assert torch.equal(y1, y2)
    np.testing.assert_allclose(y2.cpu().numpy(), oop.matvec(x.cpu().numpy()).real, atol=1e-11)


def test_device_pointers(sed, oracle):
    import torch
    built, ob, oop = both(sed, oracle, MODELS["chain24"])
    D = len(ob.reps)
    x = torch.randn(D, dtype=torch.float64, device="cuda")
    y = sed.apply(built.hamiltonian, x)
    torch.cuda.synchronize()
    np.testing.assert_allclose(y.cpu().numpy(), oop.matvec(x.cpu().numpy()).real, atol=1e-10)


def test_expectation(sed, oracle):
    built, ob, oop = both(sed, oracle, MODELS["chain16_k5_complex"])
    D = len(ob.reps)
    rng = np.random.default_rng(9)
    x = np.asfortranarray(rng.normal(size=(D, 2)) + 1j * rng.normal(size=(D, 2)))
    got = sed.expectation(built.hamiltonian, x)
    for c in range(2):
        want = np.vdot(x[:, c], oop.matvec(x[:, c]))
        assert got[c] == pytest.approx(want, rel=1e-11)


def test_hermitian_property_large(sed, oracle):
    """Size-independent check at 6x6 scale (D ~ 1.6e7): <x, H y> = <H x, y>
    and linearity, through the device-pointer entry point."""
    import torch
    from spined.model import build_model
    from _burnside import sector_dimension
    m = lattices.heisenberg_square(6)
    built = build_model(m)
    D = sed.get_number_states(built.basis)
    g = oracle.group_closure(36, m.symmetries)
    assert D == sector_dimension(g, 36, 18, 1)  # 15,804,956
    g = torch.Generator(device="cuda").manual_seed(0)
    x = torch.randn(D, dtype=torch.float64, device="cuda", generator=g)
    y = torch.randn(D, dtype=torch.float64, device="cuda", generator=g)
    hx, hy, hxy = sed.apply(built.hamiltonian, x), sed.apply(built.hamiltonian, y), sed.apply(built.hamiltonian, x + 2 * y)
    torch.cuda.synchronize()
    a = torch.dot(x, hy).item()
    b = torch.dot(hx, y).item()
    assert a == pytest.approx(b, rel=1e-10)
    assert torch.allclose(hxy, hx + 2 * hy, rtol=0, atol=1e-9)


@pytest.mark.parametrize("block", [2, 3, 5, 8, 16, 21])
def test_block_matvec_bit_identical_to_columns(sed, oracle, block):
    """Multi-column passes decode each element once for K columns; per column
    the sum is the single-column one, so the results agree bit for bit."""
    import torch
    built, ob, oop = both(sed, oracle, MODELS["chain20_j2"])
    op = built.hamiltonian
    op.prepare(L.SED_FORM_STREAM)
    D = len(ob.reps)
    x = torch.randn(block, D + 5, dtype=torch.float64, device="cuda").t()[:D]  # stride D + 5
    y = torch.zeros(block, D + 3, dtype=torch.float64, device="cuda").t()[:D]
    sed.inplace_apply(op, x, y)
    torch.cuda.synchronize()
    for c in range(block):
        yc = sed.apply(op, x[:, c].contiguous())
        torch.cuda.synchronize()
        assert torch.equal(y[:, c], yc)
    np.testing.assert_allclose(y[:, 0].cpu().numpy(), oop.matvec(x[:, 0].cpu().numpy()).real, atol=1e-11)


TABLE_MODELS = {
    "chain24": lattices.heisenberg_chain(24),
    "chain16_k8": lattices.heisenberg_chain(16, momentum=8, parity=None),   # k = pi: characters +-1
    "chain18_k9_odd": lattices.heisenberg_chain(18, momentum=9, parity=1),
    "chain14_w5": lattices.heisenberg_chain(14, hamming_weight=5),          # no spin inversion
    "square4_inv-": lattices.heisenberg_square(4, spin_inversion=-1),
    "square4_j2": lattices.heisenberg_square(4, j2=0.3),
    "ring10_nohw": lattices.Model("ring10", 10, None, 1, [(lattices.chain_translation(10), 0)],
                                  [(lattices.HEISENBERG, lattices.chain_bonds(10))]),
    "chain12_3site_weight_changing": MODELS["chain12_3site"],
    "square4_kpi": lattices.Model("sq4kpi", 16, 8, 1, [(g, 2) for g in lattices.square_symmetries(4)[:2]],
                                  [(lattices.HEISENBERG, lattices.square_bonds(4))]),
    "square4_nohw": lattices.Model("sq4nohw", 16, None, 1, [(g, 0) for g in lattices.square_symmetries(4)],
                                   [(lattices.HEISENBERG, lattices.square_bonds(4))]),
    "torus6x4_w11_j2": lattices.Model("t6x4", 24, 11, None, [(g, 0) for g in lattices.rect_translations(6, 4)],
                                      [(lattices.HEISENBERG, lattices.rect_bonds(6, 4)),
                                       ([[0.4 * v for v in r] for r in lattices.HEISENBERG],
                                        [[y * 6 + x, ((y + 1) % 4) * 6 + (x + 1) % 6] for y in range(4) for x in range(6)])]),
    "chain12_field": lattices.Model("chain12f", 12, 6, None, [(lattices.chain_translation(12), 0)],
                                    [(lattices.HEISENBERG, lattices.chain_bonds(12)),
                                     ([[0.3, 0.0], [0.0, -0.3]], [[i] for i in range(12)])]),
}


@pytest.mark.parametrize("name", list(TABLE_MODELS))
def test_orbit_table_record_bit_identical(sed, oracle, name):
    """The stream form recorded through the orbit table (a map from every word
    of the weight class to its representative) equals the one recorded by
    canonicalising every element: the same entries, so bit-identical
    matvecs; and both match the oracle."""
    import torch
    from spined.model import build_model
    m = TABLE_MODELS[name]
    lib = L.load()
    built, ob, oop = both(sed, oracle, m)
    try:
        lib.sed_set_record_mode(L.SED_RECORD_CANONICALISE)
        canon = build_model(m)
        canon.hamiltonian.prepare(L.SED_FORM_STREAM)
    finally:
        lib.sed_set_record_mode(L.SED_RECORD_AUTO)
    built.hamiltonian.prepare(L.SED_FORM_STREAM)
    assert lib.sed_operator_recorded_with_table(built.hamiltonian.ptr) == 1
    assert lib.sed_operator_recorded_with_table(canon.hamiltonian.ptr) == 0
    assert built.hamiltonian.stream_elements == canon.hamiltonian.stream_elements
    D = len(ob.reps)
    x = torch.randn(D, dtype=torch.float64, device="cuda")
    y1, y2 = torch.zeros_like(x), torch.zeros_like(x)
    sed.inplace_apply(built.hamiltonian, x, y1)
    sed.inplace_apply(canon.hamiltonian, x, y2)
    torch.cuda.synchronize()
    assert torch.equal(y1, y2)
    np.testing.assert_allclose(y1.cpu().numpy(), oop.matvec(x.cpu().numpy()).real, rtol=0,
                               atol=1e-12 * max(1.0, float(y1.abs().max())))


@pytest.mark.parametrize("name", ["chain24", "chain20_j2", "square4_j2"])
def test_fixed_point_matvec_scales_and_specials(sed, oracle, name):
    """The FP64 matvec of real operators with at most 4 distinct couplings
    accumulates u_j = round(sqrt(S_j) x_j 2^F) in int64 with F chosen per
    vector from max|x|: results match the oracle at 1e-12 of max|y| at any
    scale of x, a zero vector gives zeros, a NaN or infinity in x gives NaN
    everywhere, and entries far below max|x| are carried with an absolute
    error below 2^-55 max|x|."""
    import torch
    built, ob, oop = both(sed, oracle, MODELS[name])
    op = built.hamiltonian
    D = len(ob.reps)
    rng = np.random.default_rng(21)
    x0 = rng.normal(size=D)
    for scale in (1e-300, 1e-150, 1e-8, 1.0, 1e8, 1e150, 1e300):
        x = torch.tensor(x0 * scale, device="cuda")
        y = sed.apply(op, x).cpu().numpy()
        want = oop.matvec(x0 * scale).real
        np.testing.assert_allclose(y, want, rtol=0, atol=RTOL64 * np.abs(want).max())
    z = sed.apply(op, torch.zeros(D, dtype=torch.float64, device="cuda")).cpu().numpy()
    assert np.all(z == 0.0)
    for bad in (np.nan, np.inf):
        xb = x0.copy()
        xb[D // 2] = bad
        yb = sed.apply(op, torch.tensor(xb, device="cuda")).cpu().numpy()
        assert np.all(np.isnan(yb))
    # wide dynamic range: half the entries 1e-12 of the others
    xw = x0.copy()
    xw[::2] *= 1e-12
    yw = sed.apply(op, torch.tensor(xw, device="cuda")).cpu().numpy()
    want = oop.matvec(xw).real
    assert np.max(np.abs(yw - want)) <= 1e-13 * np.abs(xw).max() * oop.sparse().__abs__().sum(axis=1).max()
