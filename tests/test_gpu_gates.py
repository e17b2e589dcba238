"""GPU parity: gates, generators and dense matrices through the C ABI vs the oracle.

Tolerances: complex128 states within 1e-12 elementwise of the oracle;
complex64 states within 5e-6 (single-precision rounding of a unit-norm state
after one gate).
"""
import ctypes as C
import itertools

import zlib

import numpy as np
import pytest

import oracle as O
from abi import State, make_ops
from pennylane_lightning_kokkos import _native as N
from test_oracle_golden import ALL_GATES, gate_matrix, rand_state

pytestmark = pytest.mark.gpu

TOL = {N.PLK_C128: 1e-12, N.PLK_C64: 5e-6}
DTYPES = [N.PLK_C128, N.PLK_C64]


def check_gate(name, nq, wires, inverse, params, dtype, rng):
    psi = rand_state(nq, rng)
    ref = O.apply(psi.copy(), name, wires, inverse, params)
    s = State.from_array(psi, dtype)
    s.apply(name, wires, inverse, params)
    np.testing.assert_allclose(s.get(), ref, atol=TOL[dtype], rtol=0, err_msg=f"{name} {wires} inv={inverse}")


@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("name", sorted(ALL_GATES))
def test_gate_all_wire_orders(name, dtype):
    nw, npar = ALL_GATES[name]
    rng = np.random.default_rng(zlib.crc32(f"{name}/{dtype}".encode()))
    nq = nw + 1
    perms = list(itertools.permutations(range(nq), nw))
    if len(perms) > 40:
        perms = [perms[i] for i in rng.choice(len(perms), 40, replace=False)]
    for wires in perms:
        params = list(rng.uniform(0, 2 * np.pi, npar))
        for inverse in (False, True):
            check_gate(name, nq, list(wires), inverse, params, dtype, rng)


@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("name", ["PauliX", "Hadamard", "RX", "RZ", "CNOT", "CRY", "IsingXX", "IsingXY",
                                  "SingleExcitation", "SingleExcitationPlus", "DoubleExcitation",
                                  "DoubleExcitationMinus", "Toffoli", "MultiRZ", "Rot"])
def test_gate_large_state_spread_wires(name, dtype):
    # 18 qubits: targets at the highest, middle and lowest bit positions
    nw, npar = ALL_GATES[name]
    rng = np.random.default_rng(5)
    nq = 18
    for wires in ([0, 17, 9, 4][:nw], [17, 16, 15, 14][:nw], [3, 11, 0, 16][:nw], list(rng.choice(nq, nw, False))):
        check_gate(name, nq, [int(w) for w in wires], bool(rng.integers(2)), list(rng.uniform(0, 6.3, npar)), dtype,
                   rng)


GEN_GATES = ["RX", "RY", "RZ", "PhaseShift", "CRX", "CRY", "CRZ", "ControlledPhaseShift", "IsingXX", "IsingXY",
             "IsingYY", "IsingZZ", "SingleExcitation", "SingleExcitationMinus", "SingleExcitationPlus",
             "DoubleExcitation", "DoubleExcitationMinus", "DoubleExcitationPlus", "MultiRZ"]


@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("name", GEN_GATES)
def test_generator_parity(name, dtype):
    nw = ALL_GATES[name][0]
    rng = np.random.default_rng(17)
    nq = 6
    for _ in range(4):
        wires = [int(w) for w in rng.choice(nq, nw, replace=False)]
        psi = rand_state(nq, rng)
        ref = psi.copy()
        ref_scale = O.apply_generator(ref, name, wires)
        s = State.from_array(psi, dtype)
        scale = s.generator(name, wires)
        assert scale == ref_scale
        np.testing.assert_allclose(s.get(), ref, atol=TOL[dtype], rtol=0)


def test_generator_unknown_rejected():
    s = State(3)
    with pytest.raises(N.NativeError, match="Generator does not exist for Hadamard"):
        s.generator("Hadamard", [0])


def haar(dim, rng):
    z = (rng.normal(size=(dim, dim)) + 1j * rng.normal(size=(dim, dim))) / np.sqrt(2)
    q, r = np.linalg.qr(z)
    d = np.diag(r)
    return q * (d / np.abs(d))


@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("k", [1, 2, 3, 4, 5, 6])
def test_dense_matrix_parity(k, dtype):
    rng = np.random.default_rng(100 + k)
    nq = max(k + 2, 7)
    for trial in range(3):
        m = haar(1 << k, rng) if trial < 2 else rng.normal(size=(1 << k, 1 << k)) + 0j
        wires = [int(w) for w in rng.choice(nq, k, replace=False)]
        for inverse in (False, True):
            psi = rand_state(nq, rng)
            ref = O.apply_matrix(psi.copy(), m, wires, inverse)
            s = State.from_array(psi, dtype)
            s.apply_matrix(m, wires, inverse)
            scale = max(1.0, float(np.abs(m).max()) * (1 << k) / 4)
            np.testing.assert_allclose(s.get(), ref, atol=TOL[dtype] * scale, rtol=0)


@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("k", [3, 4])
def test_dense_matrix_large_state(k, dtype):
    """3- and 4-wire matrices (one group per thread, amplitudes in registers)
    on 16 qubits, with the wires at the highest, lowest and scattered bit
    positions and in unsorted order."""
    rng = np.random.default_rng(300 + k)
    nq = 16
    for wires in ([0, 1, 2, 3][:k], [15, 14, 13, 12][:k], [9, 0, 15, 4][:k], list(rng.choice(nq, k, False))):
        m = haar(1 << k, rng)
        psi = rand_state(nq, rng)
        ref = O.apply_matrix(psi.copy(), m, [int(w) for w in wires], False)
        s = State.from_array(psi, dtype)
        s.apply_matrix(m, [int(w) for w in wires])
        np.testing.assert_allclose(s.get(), ref, atol=TOL[dtype] * 4, rtol=0, err_msg=str(wires))


def test_matrix_equals_named_gate():
    # Test_StateVectorKokkos_NonParam.cpp:932-1010, on random wires of 7 qubits
    rng = np.random.default_rng(2)
    for name in ("Toffoli", "CSWAP", "DoubleExcitation", "IsingXY", "Rot"):
        nw, npar = ALL_GATES[name]
        params = list(rng.uniform(0, 6, npar))
        m = gate_matrix(name, nw, params)
        wires = [int(w) for w in rng.choice(7, nw, replace=False)]
        psi = rand_state(7, rng)
        a = State.from_array(psi).apply(name, wires, False, params).get()
        b = State.from_array(psi).apply_matrix(m, wires).get()
        np.testing.assert_allclose(a, b, atol=1e-12)


@pytest.mark.parametrize("dtype", DTYPES)
def test_apply_ops_list_matches_sequence(dtype):
    rng = np.random.default_rng(9)
    nq = 8
    ops = []
    for _ in range(60):
        name = str(rng.choice(sorted(ALL_GATES)))
        nw, npar = ALL_GATES[name]
        ops.append((name, [int(w) for w in rng.choice(nq, nw, replace=False)], bool(rng.integers(2)),
                    list(rng.uniform(0, 6.3, npar))))
    ops.append(("QubitUnitary", [2, 5], False, [], haar(4, rng)))
    psi = rand_state(nq, rng)
    ref = psi.copy()
    for op in ops:
        if len(op) > 4:
            O.apply_matrix(ref, op[4], op[1], op[2])
        else:
            O.apply(ref, *op)
    s = State.from_array(psi, dtype)
    arr, keep = make_ops(ops)
    N.check(N.lib.plk_apply_ops(s.h, arr, len(ops)))
    np.testing.assert_allclose(s.get(), ref, atol=50 * TOL[dtype], rtol=0)


def test_state_init_and_movers():
    s = State(5)
    e = np.zeros(32, complex)
    e[0] = 1
    np.testing.assert_array_equal(s.get(), e)
    N.check(N.lib.plk_state_set_basis(s.h, 7))
    e[:] = 0
    e[7] = 1
    np.testing.assert_array_equal(s.get(), e)
    import ctypes as C
    idx = np.array([1, 30], dtype=np.uint64)
    vals = np.array([0.6, 0.8j], dtype=np.complex128)
    N.check(N.lib.plk_state_set_values(s.h, idx.ctypes.data_as(C.POINTER(C.c_uint64)),
                                       vals.ctypes.data_as(C.c_void_p), 2))
    e[:] = 0
    e[1], e[30] = 0.6, 0.8j
    np.testing.assert_array_equal(s.get(), e)
    t = State(5)
    N.check(N.lib.plk_state_copy(t.h, s.h))
    np.testing.assert_array_equal(t.get(), e)
    N.check(N.lib.plk_state_axpy(t.h, 2.0, 0.5, s.h))
    np.testing.assert_allclose(t.get(), e + (2 + 0.5j) * e, atol=1e-15)
    N.check(N.lib.plk_state_reset(t.h))
    e[:] = 0
    e[0] = 1
    np.testing.assert_array_equal(t.get(), e)


@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("nq", [1, 9, 16])
def test_axpy_real_and_complex(dtype, nq):
    """y += a x (LinearAlgebraKokkos.hpp axpy_Kokkos) with a real and a
    complex coefficient."""
    rng = np.random.default_rng(70 + nq)
    x, y = rand_state(nq, rng), rand_state(nq, rng)
    tol = 1e-15 if dtype == N.PLK_C128 else 1e-6
    for a in (0.75, -1.25 + 0.5j):
        xs, ys = State.from_array(x, dtype), State.from_array(y, dtype)
        N.check(N.lib.plk_state_axpy(ys.h, a.real, complex(a).imag, xs.h))
        cast = (lambda v: v.astype(np.complex64).astype(np.complex128)) if dtype == N.PLK_C64 else (lambda v: v)
        ref = cast(y) + a * cast(x)
        np.testing.assert_allclose(ys.get(), ref, atol=tol * 4, rtol=0)


def test_invalid_arguments_are_rejected():
    s = State(3)
    with pytest.raises(N.NativeError, match="out of range"):
        s.apply("RX", [3], False, [0.1])
    with pytest.raises(N.NativeError, match="repeated wire"):
        s.apply("CNOT", [1, 1])
    with pytest.raises(N.NativeError, match="acts on 2 wires"):
        s.apply("CNOT", [0])
    with pytest.raises(N.NativeError, match="parameter"):
        s.apply("RX", [0], False, [])
    with pytest.raises(N.NativeError, match="at least one wire"):
        s.apply_matrix(np.eye(1), [])


@pytest.fixture
def dense_tc_switch():
    old = C.c_int32()
    N.check(N.lib.plk_get_dense_tensor_cores(C.byref(old)))
    yield lambda on: N.check(N.lib.plk_set_dense_tensor_cores(int(on)))
    N.check(N.lib.plk_set_dense_tensor_cores(old.value))


@pytest.mark.parametrize("k", [5, 6])
def test_dense_matrix_tensor_cores_c64(k, dense_tc_switch):
    """complex64 matrices on 5 and 6 wires: the tensor-core kernel (TF32,
    three products per step) against the CUDA-core kernel and the oracle on
    15 qubits, wires at the highest, lowest and scattered bit positions,
    unsorted; tolerance 5e-6 (single-precision rounding of the state)."""
    rng = np.random.default_rng(600 + k)
    nq = 15
    for t, wires in enumerate((list(range(k)), list(range(nq - 1, nq - 1 - k, -1)),
                               [int(w) for w in rng.choice(nq, k, False)])):
        m = haar(1 << k, rng)
        inverse = t == 2
        psi = rand_state(nq, rng)
        ref = O.apply_matrix(psi.copy(), m, wires, inverse)
        out = {}
        for on in (True, False):
            dense_tc_switch(on)
            s = State.from_array(psi, N.PLK_C64)
            s.apply_matrix(m, wires, inverse)
            out[on] = s.get()
        np.testing.assert_allclose(out[True], ref, atol=5e-6, rtol=0, err_msg=f"tensor cores {wires}")
        np.testing.assert_allclose(out[True], out[False], atol=5e-6, rtol=0, err_msg=f"tc vs cuda cores {wires}")


@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("k", [5, 7])
def test_dense_matrix_many_wires_large_state(k, dtype):
    """5- and 7-wire matrices on 13 qubits (complex128: double-float kernel,
    the 7-wire matrix read through L1/L2; complex64: tensor cores for 5 wires,
    the CUDA-core kernel for 7)."""
    rng = np.random.default_rng(700 + k)
    nq = 13
    for wires in (list(range(k)), [int(w) for w in rng.choice(nq, k, False)]):
        m = haar(1 << k, rng)
        psi = rand_state(nq, rng)
        ref = O.apply_matrix(psi.copy(), m, wires, False)
        s = State.from_array(psi, dtype)
        s.apply_matrix(m, wires, False)
        np.testing.assert_allclose(s.get(), ref, atol=TOL[dtype] * 4, rtol=0, err_msg=str(wires))
