"""GPU parity: expectation values, probabilities, CDF and sampling vs the oracle.

Tolerances: complex128 expectation values within 1e-10 of the oracle
(FP64 accumulation on both sides, different summation order); complex64
states accumulate in FP64 too, so their error is the state's single-precision
rounding (<= 1e-5 here).  Sampling is bit-exact given the same CDF and the
same uniforms; the GPU CDF is within 1e-12 of the oracle's serial scan.
"""
import ctypes as C

import numpy as np
import pytest

import known_answers as KA
import oracle as O
from abi import State, cmat, f64, i64
from pennylane_lightning_kokkos import _native as N
from test_gpu_gates import haar
from test_oracle_golden import rand_state

pytestmark = pytest.mark.gpu

ETOL = {N.PLK_C128: 1e-10, N.PLK_C64: 1e-5}
DTYPES = [N.PLK_C128, N.PLK_C64]


@pytest.mark.parametrize("dtype", DTYPES)
def test_named_expvals(dtype):
    rng = np.random.default_rng(1)
    nq = 9
    psi = rand_state(nq, rng)
    s = State.from_array(psi, dtype)
    for name in ("Identity", "PauliX", "PauliY", "PauliZ", "Hadamard"):
        for w in range(nq):
            ref = O.expval_named(psi, name, [w])
            assert abs(s.expval_named(name, [w]) - ref) < ETOL[dtype], (name, w)


@pytest.mark.parametrize("dtype", DTYPES)
def test_named_expval_batch(dtype):
    rng = np.random.default_rng(2)
    nq = 20
    psi = rand_state(nq, rng)
    s = State.from_array(psi, dtype)
    names = ["PauliZ"] * nq + ["PauliX", "Identity", "PauliY", "Hadamard"]
    wires = list(range(nq)) + [3, 0, 7, 19]
    g = np.array([N.GATE_ID[n] for n in names], dtype=np.int32)
    w, wp = i64(wires)
    out = np.zeros(len(names))
    N.check(N.lib.plk_expval_named_batch(s.h, len(names), g.ctypes.data_as(C.POINTER(C.c_int32)), wp,
                                         out.ctypes.data_as(C.POINTER(C.c_double))))
    for i, (n, ww) in enumerate(zip(names, wires)):
        assert abs(out[i] - O.expval_named(psi, n, [ww])) < ETOL[dtype]


@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("nq", [1, 3, 5, 8, 9, 10, 12, 14, 17, 22])
def test_pauliz_sets_all_sizes(nq, dtype):
    # PauliZ on every wire (each wire twice, in a shuffled order) and Identity:
    # wires whose bits fall on lanes, steps and chunks of the one-pass
    # reduction, and more values than one pass takes when nq >= 22
    rng = np.random.default_rng(100 + nq)
    psi = rand_state(nq, rng)
    s = State.from_array(psi, dtype)
    wires = list(rng.permutation(nq)) + list(range(nq)) + [0] * 3
    names = ["PauliZ"] * (2 * nq) + ["Identity"] * 3
    if nq >= 22:
        wires += list(range(nq)) * 2
        names += ["PauliZ"] * (2 * nq)
    g = np.array([N.GATE_ID[n] for n in names], dtype=np.int32)
    w, wp = i64(wires)
    out = np.zeros(len(names))
    N.check(N.lib.plk_expval_named_batch(s.h, len(names), g.ctypes.data_as(C.POINTER(C.c_int32)), wp,
                                         out.ctypes.data_as(C.POINTER(C.c_double))))
    for i, (n, ww) in enumerate(zip(names, wires)):
        assert abs(out[i] - O.expval_named(psi, n, [int(ww)])) < ETOL[dtype], (n, ww)


@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("k", [1, 2, 3, 4])
def test_matrix_expval(k, dtype):
    rng = np.random.default_rng(10 + k)
    nq = 8
    psi = rand_state(nq, rng)
    s = State.from_array(psi, dtype)
    for _ in range(3):
        m = rng.normal(size=(1 << k, 1 << k)) + 1j * rng.normal(size=(1 << k, 1 << k))
        m = m + m.conj().T
        wires = [int(x) for x in rng.choice(nq, k, replace=False)]
        ref = O.expval_matrix(psi, m, wires)
        assert abs(s.expval_matrix(m, wires) - ref) < ETOL[dtype] * 10 * (1 << k)


@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("k", [1, 2, 3])
def test_matrix_expval_general_matrix(k, dtype):
    """Re<psi|M|psi> of a non-Hermitian matrix (the kernels evaluate the
    Hermitian part) on 14 qubits, wires at both ends and scattered."""
    rng = np.random.default_rng(40 + k)
    nq = 14
    psi = rand_state(nq, rng)
    s = State.from_array(psi, dtype)
    for wires in ([0, 1, 2][:k], [13, 12, 11][:k], [int(x) for x in rng.choice(nq, k, replace=False)]):
        m = rng.normal(size=(1 << k, 1 << k)) + 1j * rng.normal(size=(1 << k, 1 << k))
        ref = O.expval_matrix(psi, m, wires)
        assert abs(s.expval_matrix(m, wires) - ref) < ETOL[dtype] * 10 * (1 << k), wires


def test_expval_known_answers_gpu():
    s = State.from_array(KA.INI_3Q_C)
    assert s.expval_matrix(KA.HERMITIAN_3Q_MATRIX, [0, 1, 2]) == pytest.approx(KA.EXPVAL_HERMITIAN_3Q, rel=1e-7)
    d, dp = cmat(KA.SPARSE_VALUES)
    ind, indp = i64(KA.SPARSE_INDICES)
    ptr, ptrp = i64(KA.SPARSE_INDPTR)
    out = C.c_double()
    N.check(N.lib.plk_expval_sparse(s.h, dp, indp, ptrp, 8, 16, C.byref(out)))
    assert out.value == pytest.approx(KA.EXPVAL_SPARSE, rel=1e-7)


def pauli_obs(words):
    terms = []
    for c, wires, letters in words:
        factors = [("named", {"X": "PauliX", "Y": "PauliY", "Z": "PauliZ"}[l], [w]) for w, l in zip(wires, letters)
                   if l != "I"]
        terms.append(("tensor", factors) if factors else ("named", "Identity", [0]))
    return ("hamiltonian", [w[0] for w in words], terms)


def random_words(nq, count, rng, max_weight=4):
    words = []
    for _ in range(count):
        wt = int(rng.integers(1, max_weight + 1))
        wires = [int(x) for x in rng.choice(nq, wt, replace=False)]
        letters = "".join(rng.choice(list("XYZ"), wt))
        words.append((float(rng.normal()), wires, letters))
    return words


def pauli_args(words):
    c, cp = f64([w[0] for w in words])
    offs = np.cumsum([0] + [len(w[1]) for w in words])
    o, op = i64(offs)
    ww, wp = i64([x for w in words for x in w[1]] or [0])
    letters = "".join(w[2] for w in words).encode()
    return (c, o, ww, letters), (cp, op, wp, letters)


@pytest.mark.parametrize("dtype", DTYPES)
def test_pauli_sum_expval(dtype):
    rng = np.random.default_rng(3)
    nq = 10
    psi = rand_state(nq, rng)
    words = random_words(nq, 40, rng) + [(0.7, [2, 5], "ZZ"), (-0.3, [1], "I"), (0.25, [4, 1, 8], "YYY")]
    ref = O.expval_observable(psi, pauli_obs(words))
    s = State.from_array(psi, dtype)
    keep, (cp, op, wp, letters) = pauli_args(words)
    out = C.c_double()
    N.check(N.lib.plk_expval_pauli_sum(s.h, len(words), cp, op, wp, letters, C.byref(out)))
    assert abs(out.value - ref) < ETOL[dtype] * 20


SINGLE_WORDS = [(0.9, [0], "X"), (-0.4, [12], "Y"), (1.3, [5], "Z"), (0.6, [0, 12], "XY"), (-1.1, [12, 0], "YY"),
                (0.8, [3, 7], "XZ"), (0.5, [7, 3], "ZY"), (-0.7, [1, 6, 11], "YXZ"), (0.3, [2, 9, 4, 10], "YYYX"),
                (1.2, [11, 10], "ZZ")]


@pytest.mark.parametrize("dtype", DTYPES)
def test_pauli_words_one_at_a_time(dtype):
    """Each word on its own (one-term X groups: real and imaginary parts,
    the pair's top bit low and high, diagonal words), on 13 qubits so that
    the application kernel spans several 2048-amplitude tiles."""
    rng = np.random.default_rng(31)
    nq = 13
    psi = rand_state(nq, rng)
    s = State.from_array(psi, dtype)
    ptol = 1e-12 if dtype == N.PLK_C128 else 2e-5
    for word in SINGLE_WORDS:
        ref = O.expval_observable(psi, pauli_obs([word]))
        keep, (cp, op, wp, letters) = pauli_args([word])
        out = C.c_double()
        N.check(N.lib.plk_expval_pauli_sum(s.h, 1, cp, op, wp, letters, C.byref(out)))
        assert abs(out.value - ref) < ETOL[dtype] * 4, word
        hout = State(nq, dtype)
        N.check(N.lib.plk_apply_pauli_sum(hout.h, s.h, 1, cp, op, wp, letters))
        np.testing.assert_allclose(hout.get(), O.apply_observable(psi.copy(), pauli_obs([word])), atol=ptol * 4,
                                   err_msg=str(word))


@pytest.mark.parametrize("dtype", DTYPES)
def test_apply_pauli_sum(dtype):
    rng = np.random.default_rng(4)
    nq = 9
    psi = rand_state(nq, rng)
    words = random_words(nq, 25, rng)
    ref = O.apply_observable(psi.copy(), pauli_obs(words))
    s = State.from_array(psi, dtype)
    out = State(nq, dtype)
    keep, (cp, op, wp, letters) = pauli_args(words)
    N.check(N.lib.plk_apply_pauli_sum(out.h, s.h, len(words), cp, op, wp, letters))
    tol = 1e-12 if dtype == N.PLK_C128 else 2e-5
    np.testing.assert_allclose(out.get(), ref, atol=tol * 10)


def test_inner_product_and_spmv():
    rng = np.random.default_rng(5)
    a, b = rand_state(8, rng), rand_state(8, rng)
    x, y = State.from_array(a), State.from_array(b)
    re, im = C.c_double(), C.c_double()
    N.check(N.lib.plk_inner_product(x.h, y.h, C.byref(re), C.byref(im)))
    ref = np.vdot(a, b)
    assert abs(re.value - ref.real) < 1e-13 and abs(im.value - ref.imag) < 1e-13
    # SpMV with the reference's known answer (Test_LinearAlgebra.cpp:10-52)
    xs = State.from_array(KA.SPMV_X)
    ys = State(3)
    d, dp = cmat(KA.SPMV_VALUES)
    ind, indp = i64(KA.SPARSE_INDICES)
    ptr, ptrp = i64(KA.SPARSE_INDPTR)
    N.check(N.lib.plk_spmv(ys.h, xs.h, dp, indp, ptrp, 8, 16))
    np.testing.assert_allclose(ys.get(), KA.SPMV_RESULT, atol=1e-12)


@pytest.mark.parametrize("wires,expected", KA.PROBS_CASES)
def test_probs_known_answers_gpu(wires, expected):
    s = State(3)
    for name, w, inv, p in KA.PROBS_INIT_OPS:
        s.apply(name, w, inv, p)
    np.testing.assert_allclose(s.probs(wires), expected, atol=KA.PROBS_MARGIN)


@pytest.mark.parametrize("dtype", DTYPES)
def test_probs_random_wires(dtype):
    rng = np.random.default_rng(6)
    nq = 14
    psi = rand_state(nq, rng)
    s = State.from_array(psi, dtype)
    tol = 1e-13 if dtype == N.PLK_C128 else 1e-6
    np.testing.assert_allclose(s.probs(), O.probs(psi), atol=tol)
    for m in (1, 2, 3, 5, 8, 12, 13, 14):
        wires = [int(x) for x in rng.permutation(nq)[:m]]
        np.testing.assert_allclose(s.probs(wires), O.probs(psi, wires), atol=tol * 4, err_msg=str(wires))


@pytest.mark.parametrize("dtype", DTYPES)
def test_probs_marginal_layouts(dtype):
    """Marginals whose measured bits are the highest, the lowest, interleaved
    or scattered, with many amplitudes per bin (chunked bins) and with fewer
    than 32 amplitudes per bin (one thread per bin); repeated calls give the
    same bits (fixed summation order)."""
    rng = np.random.default_rng(16)
    nq = 20
    psi = rand_state(nq, rng)
    s = State.from_array(psi, dtype)
    tol = 1e-13 if dtype == N.PLK_C128 else 1e-6
    ref_psi = s.get().astype(np.complex128)
    cases = [[0], [nq - 1], [0, 1, 2], [nq - 3, nq - 2, nq - 1], [nq - 1, 0], list(range(0, nq, 2)),
             list(range(13)), list(range(nq - 13, nq)), [int(x) for x in rng.permutation(nq)[:14]],
             [int(x) for x in rng.permutation(nq)[:15]], [int(x) for x in rng.permutation(nq)[:17]],
             [int(x) for x in rng.permutation(nq)]]
    for wires in cases:
        got = s.probs(wires)
        np.testing.assert_allclose(got, O.probs(ref_psi, wires), atol=tol, rtol=0, err_msg=str(wires))
        np.testing.assert_array_equal(got, s.probs(wires))


@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("nq", [1, 5, 11, 12, 13, 20])
def test_cdf_sizes(dtype, nq):
    """Exclusive CDF for states smaller than one 4096-amplitude tile, exactly
    one tile, a few tiles and many tiles."""
    rng = np.random.default_rng(100 + nq)
    psi = rand_state(nq, rng)
    s = State.from_array(psi, dtype)
    n = 1 << nq
    cdf = np.empty(n)
    N.check(N.lib.plk_cdf(s.h, cdf.ctypes.data_as(C.POINTER(C.c_double))))
    ref = O.cdf_exclusive(O.probs(s.get().astype(np.complex128)))
    np.testing.assert_allclose(cdf, ref, atol=1e-12, rtol=0)
    assert cdf[0] == 0.0


@pytest.mark.parametrize("dtype", DTYPES)
def test_cdf_and_sampling_bit_exact(dtype):
    rng = np.random.default_rng(7)
    nq = 16
    psi = rand_state(nq, rng)
    s = State.from_array(psi, dtype)
    n = 1 << nq
    cdf = np.empty(n)
    N.check(N.lib.plk_cdf(s.h, cdf.ctypes.data_as(C.POINTER(C.c_double))))
    ref_cdf = O.cdf_exclusive(O.probs(s.get().astype(np.complex128)))
    np.testing.assert_allclose(cdf, ref_cdf, atol=1e-12, rtol=0)
    # identical CDF + identical uniforms -> identical indices (incl. edge draws)
    u = np.concatenate([rng.random(20000), [0.0, cdf[1], cdf[1] + 1e-17, cdf[n // 2], cdf[-1], 1.0 - 1e-16]])
    out = np.empty((u.size, nq), dtype=np.int64)
    cc, ccp = f64(ref_cdf)
    uu, up = f64(u)
    N.check(N.lib.plk_search_cdf(ccp, n, nq, up, u.size, out.ctypes.data_as(C.POINTER(C.c_int64)), 0))
    np.testing.assert_array_equal(out, O.sample_from_uniforms(ref_cdf, nq, u))
    # through the state: its own CDF and the same uniforms
    out2 = np.empty((u.size, nq), dtype=np.int64)
    N.check(N.lib.plk_sample_from_uniforms(s.h, up, u.size, out2.ctypes.data_as(C.POINTER(C.c_int64))))
    np.testing.assert_array_equal(out2, O.sample_from_uniforms(cdf, nq, u))


def test_generate_samples_histogram_and_determinism():
    # Test_StateVectorKokkos_Param.cpp:1325-1394 (margin 0.05 over 100000 shots)
    s = State(3)
    for name, w, inv, p in KA.PROBS_INIT_OPS:
        s.apply(name, w, inv, p)
    shots = KA.SAMPLE_SHOTS
    a = np.empty((shots, 3), dtype=np.int64)
    b = np.empty((shots, 3), dtype=np.int64)
    N.check(N.lib.plk_generate_samples(s.h, shots, 5374857, a.ctypes.data_as(C.POINTER(C.c_int64))))
    N.check(N.lib.plk_generate_samples(s.h, shots, 5374857, b.ctypes.data_as(C.POINTER(C.c_int64))))
    np.testing.assert_array_equal(a, b)
    hist = np.bincount(a @ np.array([4, 2, 1]), minlength=8) / shots
    np.testing.assert_allclose(hist, KA.PROBS_CASES[0][1], atol=KA.SAMPLE_MARGIN)
    # a much tighter statistical check: 5 sigma of a binomial
    p = np.array(KA.PROBS_CASES[0][1])
    assert np.all(np.abs(hist - p) < 5 * np.sqrt(p * (1 - p) / shots) + 1e-9)
