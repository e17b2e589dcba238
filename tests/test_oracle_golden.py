"""Pin the CPU oracle to the reference's own known answers (no GPU needed).

Each test names the reference test it restates; the values live in
``tests/golden/known_answers.py`` with file:line citations.
"""
import math

import zlib

import numpy as np
import pytest

import known_answers as KA
import oracle as O

ALL_GATES = {
    # name: (num wires, num params)
    "PauliX": (1, 0), "PauliY": (1, 0), "PauliZ": (1, 0), "Hadamard": (1, 0), "S": (1, 0), "T": (1, 0),
    "PhaseShift": (1, 1), "RX": (1, 1), "RY": (1, 1), "RZ": (1, 1), "Rot": (1, 3),
    "CNOT": (2, 0), "CY": (2, 0), "CZ": (2, 0), "SWAP": (2, 0), "ControlledPhaseShift": (2, 1),
    "CRX": (2, 1), "CRY": (2, 1), "CRZ": (2, 1), "CRot": (2, 3), "IsingXX": (2, 1), "IsingXY": (2, 1),
    "IsingYY": (2, 1), "IsingZZ": (2, 1), "SingleExcitation": (2, 1), "SingleExcitationMinus": (2, 1),
    "SingleExcitationPlus": (2, 1), "CSWAP": (3, 0), "Toffoli": (3, 0), "DoubleExcitation": (4, 1),
    "DoubleExcitationMinus": (4, 1), "DoubleExcitationPlus": (4, 1), "MultiRZ": (3, 1),
}


def rand_state(nq, rng):
    v = rng.normal(size=1 << nq) + 1j * rng.normal(size=1 << nq)
    return (v / np.linalg.norm(v)).astype(np.complex128)


def state_from(init, nq):
    if init is None:
        return O.zero_state(nq)
    return np.array(init, dtype=np.complex128)


@pytest.mark.parametrize("case", sorted(KA.GATE_CASES))
def test_gate_known_answers(case):
    init, nq, ops, expected, tol = KA.GATE_CASES[case]
    sv = state_from(init, nq)
    O.run_ops(sv, ops)
    np.testing.assert_allclose(sv, np.array(expected), rtol=tol, atol=tol)


def rot_matrix(phi, theta, omega):
    c, s = math.cos(theta / 2), math.sin(theta / 2)
    return np.array([[np.exp(-0.5j * (phi + omega)) * c, -np.exp(0.5j * (phi - omega)) * s],
                     [np.exp(-0.5j * (phi - omega)) * s, np.exp(0.5j * (phi + omega)) * c]])


def test_crot_known_answer():
    # Test_StateVectorKokkos_Param.cpp:461-506: CRot(0.3, 0.8, 2.4) on |100>
    angles = [0.3, 0.8, 2.4]
    r = rot_matrix(*angles)
    sv = O.zero_state(3)
    O.apply(sv, "PauliX", [0])
    O.apply(sv, "CRot", [0, 1], False, angles)
    exp = np.zeros(8, dtype=complex)
    exp[4], exp[6] = r[0, 0], r[1, 0]
    np.testing.assert_allclose(sv, exp, atol=1e-12)


@pytest.mark.parametrize("name", sorted(KA.GENERATOR_WIRES))
def test_generator_matches_finite_difference(name):
    # Test_StateVectorKokkos_Generator.cpp: d/dtheta U|psi> = i*scale*G|psi>
    ep, margin = KA.GENERATOR_FD
    wires = KA.GENERATOR_WIRES[name]
    psi = np.array(KA.INI_4Q_A, dtype=np.complex128)
    g = psi.copy()
    scale = O.apply_generator(g, name, wires)
    p, m = psi.copy(), psi.copy()
    O.apply(p, name, wires, False, [ep])
    O.apply(m, name, wires, False, [-ep])
    fd = 0.5 * (p - m) / ep
    np.testing.assert_allclose(-scale * g.imag, fd.real, atol=margin)
    np.testing.assert_allclose(scale * g.real, fd.imag, atol=margin)


@pytest.mark.parametrize("wires,expected", KA.PROBS_CASES)
def test_probs_known_answers(wires, expected):
    sv = O.run_ops(O.zero_state(3), KA.PROBS_INIT_OPS)
    np.testing.assert_allclose(O.probs(sv, wires), expected, atol=KA.PROBS_MARGIN)


def test_sampling_histogram():
    # Test_StateVectorKokkos_Param.cpp:1325-1394 with numpy uniforms in place
    # of the Kokkos XorShift64 pool.
    sv = O.run_ops(O.zero_state(3), KA.PROBS_INIT_OPS)
    cdf = O.cdf_exclusive(O.probs(sv))
    u = np.random.default_rng(7).random(KA.SAMPLE_SHOTS)
    bits = O.sample_from_uniforms(cdf, 3, u)
    idx = bits @ (1 << np.arange(2, -1, -1))
    hist = np.bincount(idx, minlength=8) / KA.SAMPLE_SHOTS
    np.testing.assert_allclose(hist, KA.PROBS_CASES[0][1], atol=KA.SAMPLE_MARGIN)


def test_sampler_edge_cases():
    # index 0 when U <= cdf[1]; the last index when U lands in the final bin;
    # cdf[N] is taken as 1 (MeasuresFunctors.hpp:94-112).
    p = np.array([0.25, 0.0, 0.5, 0.25])
    cdf = O.cdf_exclusive(p)
    u = np.array([0.0, 0.25, 0.2500001, 0.75, 0.7500001, 1.0])
    idx = O.sample_from_uniforms(cdf, 2, u) @ np.array([2, 1])
    assert list(idx) == [0, 0, 2, 2, 3, 3]


def test_expval_known_answers():
    sv = np.array(KA.INI_3Q_C, dtype=np.complex128)
    # Test_StateVectorKokkos_Expval.cpp:366-421
    assert O.expval_matrix(sv, KA.HERMITIAN_3Q_MATRIX, [0, 1, 2]) == pytest.approx(KA.EXPVAL_HERMITIAN_3Q, rel=1e-7)
    # :423-447
    assert O.expval_sparse(sv, KA.SPARSE_VALUES, KA.SPARSE_INDICES, KA.SPARSE_INDPTR) == pytest.approx(
        KA.EXPVAL_SPARSE, rel=1e-7)
    # :449-469
    ham = ("hamiltonian", [0.3, 0.5], [("named", "PauliX", [0]), ("named", "PauliZ", [1])])
    assert O.expval_observable(sv, ham) == pytest.approx(KA.EXPVAL_HAMILTONIAN, rel=1.2e-5)
    # :471-491
    ten = ("tensor", [("named", "PauliX", [0]), ("named", "PauliZ", [1])])
    assert O.expval_observable(sv, ten) == pytest.approx(KA.EXPVAL_TENSOR, rel=1.2e-5)


def test_linear_algebra_known_answers():
    # Test_LinearAlgebra.cpp:10-52 and :53-90
    x = np.array(KA.SPMV_X, dtype=np.complex128)
    y = O.spmv(x, KA.SPMV_VALUES, KA.SPARSE_INDICES, KA.SPARSE_INDPTR)
    np.testing.assert_allclose(y, KA.SPMV_RESULT, atol=1e-12)
    yy = np.array(KA.AXPY_Y, dtype=np.complex128)
    O.axpy(KA.AXPY_ALPHA, np.array(KA.AXPY_X, dtype=np.complex128), yy)
    np.testing.assert_allclose(yy, KA.AXPY_RESULT, atol=1e-12)


def test_variance_known_answers():
    sv = O.run_ops(O.zero_state(2), KA.VAR_2Q_OPS)
    for obs, exp in KA.VAR_NAMED:
        assert O.var_observable(sv, obs) == pytest.approx(exp, rel=1.2e-5)
    sv3 = O.run_ops(O.zero_state(3), KA.VAR_3Q_OPS)
    herm = ("hermitian", KA.VAR_HERMITIAN_MATRIX, [0, 2])
    assert O.var_observable(sv3, herm) == pytest.approx(KA.VAR_HERMITIAN, rel=1.2e-5)
    svt = O.run_ops(O.zero_state(3), KA.VAR_TENSOR_OPS)
    ten = ("tensor", [("named", "PauliX", [0]), ("named", "PauliZ", [1])])
    assert O.var_observable(svt, ten) == pytest.approx(KA.VAR_TENSOR, rel=1.2e-5)
    svh = np.array(KA.INI_3Q_C, dtype=np.complex128)
    ham = ("hamiltonian", [0.3, 0.5], [("named", "PauliX", [0]), ("named", "PauliZ", [1])])
    assert O.var_observable(svh, ham) == pytest.approx(KA.VAR_HAMILTONIAN, rel=1.2e-5)


@pytest.mark.parametrize("case", sorted(KA.ADJOINT_CASES))
def test_adjoint_known_answers(case):
    init, nq, ops, obs, tp, expected, margin = KA.ADJOINT_CASES[case]
    sv = O.run_ops(state_from(init, nq), ops)
    jac = O.adjoint_jacobian(sv, obs, ops, tp)
    for i, row in enumerate(expected):
        for j, e in enumerate(row):
            if e is not None:
                assert jac[i, j] == pytest.approx(e, abs=margin), (i, j, jac)


def test_adjoint_hermitian_equals_tensor():
    nq, ops, ten, herm, tp, margin = KA.ADJOINT_HERMITIAN_EQ_TENSOR
    sv = O.run_ops(O.zero_state(nq), ops)
    np.testing.assert_allclose(O.adjoint_jacobian(sv, [ten], ops, tp),
                               O.adjoint_jacobian(sv, [herm], ops, tp), atol=margin)


def gate_matrix(name, nw, params, inverse=False):
    """Dense matrix of a named gate on wires [0..nw-1], built column by column
    with the oracle itself (row index: wire 0 most significant)."""
    dim = 1 << nw
    m = np.zeros((dim, dim), dtype=np.complex128)
    for col in range(dim):
        e = np.zeros(dim, dtype=np.complex128)
        e[col] = 1
        O.apply(e, name, list(range(nw)), inverse, params)
        m[:, col] = e
    return m


@pytest.mark.parametrize("name", sorted(ALL_GATES))
def test_gates_unitary_and_inverse(name):
    nw, npar = ALL_GATES[name]
    rng = np.random.default_rng(zlib.crc32(name.encode()))
    params = list(rng.uniform(0, 2 * np.pi, npar))
    m = gate_matrix(name, nw, params)
    np.testing.assert_allclose(m.conj().T @ m, np.eye(1 << nw), atol=1e-12)
    mi = gate_matrix(name, nw, params, inverse=True)
    np.testing.assert_allclose(mi, m.conj().T, atol=1e-12)


@pytest.mark.parametrize("name", ["Hadamard", "RX", "Rot", "CNOT", "CRY", "IsingXY", "CSWAP", "Toffoli",
                                  "DoubleExcitation", "MultiRZ"])
def test_matrix_apply_equals_named_gate(name):
    # Test_StateVectorKokkos_NonParam.cpp:932-1010 pattern, on random wire orders
    nw, npar = ALL_GATES[name]
    rng = np.random.default_rng(3)
    params = list(rng.uniform(0, 2 * np.pi, npar))
    m = gate_matrix(name, nw, params)
    nq = 6
    for _ in range(6):
        wires = list(rng.choice(nq, size=nw, replace=False))
        psi = rand_state(nq, rng)
        a, b = psi.copy(), psi.copy()
        O.apply(a, name, wires, False, params)
        O.apply_matrix(b, m, wires)
        np.testing.assert_allclose(a, b, atol=1e-12)
        c = psi.copy()
        O.apply_matrix(c, m, wires, inverse=True)
        O.apply(c, name, wires, False, params)
        np.testing.assert_allclose(c, psi, atol=1e-12)


def test_reference_multiqubit_index_map_defect():
    """multiQubitOpFunctor (GateFunctors.hpp:232-252) places amplitudes by
    sequential bit swaps.  It agrees with the documented semantics when the
    target bits lie above the low k bits (and on the reference's own 3-qubit
    test layout), and departs from it otherwise.  The product follows the
    documented semantics."""
    rng = np.random.default_rng(11)
    m = gate_matrix("Toffoli", 3, [])
    u = np.linalg.qr(rng.normal(size=(8, 8)) + 1j * rng.normal(size=(8, 8)))[0]
    for mat in (m, u):
        for wires, nq in (([0, 1, 2], 3), ([0, 1, 2], 6), ([1, 0, 2], 6), ([2, 0, 1], 7)):
            psi = rand_state(nq, rng)
            a, b = psi.copy(), psi.copy()
            O.apply_matrix(a, mat, wires)
            O.apply_matrix(b, mat, wires, refmap=True)
            np.testing.assert_allclose(a, b, atol=1e-12)
    psi = rand_state(4, rng)
    a, b = psi.copy(), psi.copy()
    O.apply_matrix(a, u, [3, 1, 0])
    O.apply_matrix(b, u, [3, 1, 0], refmap=True)
    assert np.max(np.abs(a - b)) > 1e-3


def test_adjoint_matches_central_differences():
    """Adjoint Jacobian of a seeded RY/RZ + CNOT-ladder ansatz against central
    finite differences (h = 1e-6) of the PauliZ/Hamiltonian expectation."""
    rng = np.random.default_rng(4)
    nq, layers = 5, 3
    ops = []
    for _ in range(layers):
        for w in range(nq):
            ops.append(("RY", [w], False, [rng.uniform(0, 2 * np.pi)]))
            ops.append(("RZ", [w], False, [rng.uniform(0, 2 * np.pi)]))
        for w in range(nq - 1):
            ops.append(("CNOT", [w, w + 1], False, []))
    ham = ("hamiltonian", [0.4, -1.1, 0.7],
           [("named", "PauliZ", [0]), ("tensor", [("named", "PauliX", [1]), ("named", "PauliY", [3])]),
            ("named", "PauliZ", [4])])
    sv = O.run_ops(O.zero_state(nq), ops)
    npar = sum(1 for o in ops if o[3])
    jac = O.adjoint_jacobian(sv, [ham], ops, list(range(npar)))[0]
    h, k = 1e-6, 0
    for i, (name, w, inv, p) in enumerate(ops):
        if not p:
            continue
        vals = []
        for d in (h, -h):
            ops2 = list(ops)
            ops2[i] = (name, w, inv, [p[0] + d])
            vals.append(O.expval_observable(O.run_ops(O.zero_state(nq), ops2), ham))
        assert jac[k] == pytest.approx((vals[0] - vals[1]) / (2 * h), abs=1e-7)
        k += 1


def test_multirz_on_many_wires_matches_formula():
    """MultiRZ acts on any number of wires: exp(-i theta/2 Z...Z), a phase by
    the parity of the selected bits (multiRZFunctor, GateFunctors.hpp:2132-2170)."""
    rng = np.random.default_rng(7)
    for nq in (9, 12, 14):
        for k in (1, 5, nq):
            wires = [int(w) for w in rng.permutation(nq)[:k]]
            th = float(rng.uniform(-3, 3))
            psi = rng.normal(size=1 << nq) + 1j * rng.normal(size=1 << nq)
            mask = sum(1 << (nq - 1 - w) for w in wires)
            par = np.array([bin(i & mask).count("1") & 1 for i in range(1 << nq)])
            for inv in (False, True):
                ph = np.where(par, np.exp(1j * th / 2), np.exp(-1j * th / 2))
                ref = psi * (np.conj(ph) if inv else ph)
                out = psi.copy()
                O.apply(out, "MultiRZ", wires, inv, [th])
                np.testing.assert_allclose(out, ref, atol=1e-14)
                g = psi.copy()
                O.apply_generator(g, "MultiRZ", wires)
                np.testing.assert_allclose(g, psi * np.where(par, -1.0, 1.0), atol=1e-15)
