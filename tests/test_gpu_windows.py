"""GPU: register-window sweeps over one state (complex64 op lists and
one-observable adjoint Jacobians) against the op-at-a-time path and the oracle.

Tolerances: complex64 states within 5e-6 of the op-at-a-time path and of the
FP64 oracle, Jacobians within 1e-4 of the oracle and 2e-5 of the op-at-a-time
path; complex128 (double-float windows) states within 1e-12 and Jacobians
within 1e-10 of the oracle; window results are bitwise reproducible.
"""
import ctypes as C

import numpy as np
import pytest

import oracle as O
from abi import State, i64, make_ops
from pennylane_lightning_kokkos import _native as N
from test_gpu_adjoint import gpu_adjoint, random_circuit
from test_oracle_golden import ALL_GATES

pytestmark = pytest.mark.gpu


@pytest.fixture
def window_switch():
    old = C.c_int32()
    N.check(N.lib.plk_get_window_path(C.byref(old)))
    yield lambda on: N.check(N.lib.plk_set_window_path(int(on)))
    N.check(N.lib.plk_set_window_path(old.value))


def run_forward(nq, ops, dtype=N.PLK_C64):
    s = State(nq, dtype)
    arr, keep = make_ops(ops)
    N.check(N.lib.plk_apply_ops(s.h, arr, len(ops)))
    out = s.get()
    s.close()
    return out


def circuit_with_everything(nq, nops, rng):
    from pennylane_lightning_kokkos.circuits import haar_unitary

    ops = []
    for _ in range(nops):
        r = rng.random()
        if r < 0.1:
            k = int(rng.integers(1, 5))
            ops.append(("Matrix", [int(w) for w in rng.choice(nq, k, replace=False)], bool(rng.integers(2)), [],
                        haar_unitary(1 << k, rng)))
        elif r < 0.2:
            k = int(rng.integers(1, nq + 1))
            ops.append(("MultiRZ", [int(w) for w in rng.choice(nq, k, replace=False)], bool(rng.integers(2)),
                        [float(rng.uniform(0, 6))]))
        else:
            name = str(rng.choice(sorted(ALL_GATES)))
            nw, npar = ALL_GATES[name]
            if nw < 0:
                continue
            ops.append((name, [int(w) for w in rng.choice(nq, nw, replace=False)], bool(rng.integers(2)),
                        list(rng.uniform(0, 2 * np.pi, npar))))
    return ops


def oracle_forward(nq, ops):
    psi = O.zero_state(nq)
    for op in ops:
        if op[0] == "Matrix":
            O.apply_matrix(psi, op[4], op[1], op[2])
        else:
            O.apply(psi, op[0], op[1], op[2], op[3])
    return psi


STOL = {N.PLK_C64: 5e-6, N.PLK_C128: 1e-12}


@pytest.mark.parametrize("dtype", [N.PLK_C64, N.PLK_C128])
@pytest.mark.parametrize("nq", [6, 9, 12])
def test_window_forward_matches_per_op_and_oracle(nq, dtype, window_switch):
    rng = np.random.default_rng(100 + nq)
    ops = circuit_with_everything(nq, 120, rng)
    window_switch(True)
    a = run_forward(nq, ops, dtype)
    b = run_forward(nq, ops, dtype)
    window_switch(False)
    c = run_forward(nq, ops, dtype)
    np.testing.assert_array_equal(a, b)
    np.testing.assert_allclose(a, c, atol=STOL[dtype], rtol=0)
    np.testing.assert_allclose(a, oracle_forward(nq, ops), atol=STOL[dtype], rtol=0)


def test_window_forward_layered_ansatz(window_switch):
    from pennylane_lightning_kokkos.circuits import hardware_efficient_ansatz

    nq = 14
    ops = hardware_efficient_ansatz(nq, 6, seed=9, rotations=("RX", "RY", "RZ"))
    window_switch(True)
    a = run_forward(nq, ops)
    np.testing.assert_allclose(a, O.run_ops(O.zero_state(nq), ops), atol=5e-6, rtol=0)


@pytest.mark.parametrize("seed", [0, 1, 2, 3])
def test_window_adjoint_c128_matches_oracle(seed, window_switch):
    rng = np.random.default_rng(50 + seed)
    nq = 7 + seed
    ops = random_circuit(nq, 80, rng)
    npar = sum(1 for o in ops if o[3])
    trainable = sorted(int(x) for x in rng.choice(npar, max(1, npar * 2 // 3), replace=False))
    obs = [("hamiltonian", [0.7, -0.4, 1.1],
            [("named", "PauliZ", [1]), ("tensor", [("named", "PauliX", [0]), ("named", "PauliY", [3])]),
             ("named", "PauliX", [nq - 1])])]
    psi = O.run_ops(O.zero_state(nq), ops)
    ref = O.adjoint_jacobian(psi, obs, ops, trainable)
    window_switch(True)
    jw = gpu_adjoint(psi, obs, ops, trainable, N.PLK_C128)
    np.testing.assert_allclose(jw, ref, atol=1e-10, rtol=0)


@pytest.mark.parametrize("seed", [0, 1, 2, 3])
def test_window_adjoint_matches_oracle(seed, window_switch):
    rng = np.random.default_rng(seed)
    nq = 8 + seed
    ops = random_circuit(nq, 80, rng)
    npar = sum(1 for o in ops if o[3])
    trainable = sorted(int(x) for x in rng.choice(npar, max(1, npar * 2 // 3), replace=False))
    obs = [("hamiltonian", [0.7, -0.4, 1.1],
            [("named", "PauliZ", [1]), ("tensor", [("named", "PauliX", [0]), ("named", "PauliY", [3])]),
             ("named", "PauliX", [nq - 1])])]
    psi = O.run_ops(O.zero_state(nq), ops)
    ref = O.adjoint_jacobian(psi, obs, ops, trainable)
    window_switch(True)
    jw = gpu_adjoint(psi, obs, ops, trainable, N.PLK_C64)
    jw2 = gpu_adjoint(psi, obs, ops, trainable, N.PLK_C64)
    window_switch(False)
    jp = gpu_adjoint(psi, obs, ops, trainable, N.PLK_C64)
    np.testing.assert_array_equal(jw, jw2)
    np.testing.assert_allclose(jw, ref, atol=1e-4, rtol=0)
    np.testing.assert_allclose(jw, jp, atol=2e-5, rtol=0)


def test_window_adjoint_matrices_and_multirz(window_switch):
    """Non-trainable matrix ops and trainable MultiRZ on many wires."""
    from pennylane_lightning_kokkos.circuits import haar_unitary

    rng = np.random.default_rng(5)
    nq = 10
    ops = []
    for k in range(30):
        if k % 7 == 3:
            kk = int(rng.integers(1, 5))
            ops.append(("Matrix", [int(w) for w in rng.choice(nq, kk, replace=False)], bool(rng.integers(2)), [],
                        haar_unitary(1 << kk, rng)))
        elif k % 5 == 0:
            ops.append(("MultiRZ", [int(w) for w in rng.choice(nq, 6, replace=False)], bool(rng.integers(2)),
                        [float(rng.uniform(0, 6))]))
        else:
            ops.append(("RY", [k % nq], False, [float(rng.uniform(0, 6))]))
            ops.append(("CNOT", [k % nq, (k + 3) % nq], False, []))
    npar = sum(1 for o in ops if o[3])
    psi = oracle_forward(nq, ops)
    obs = [("named", "PauliZ", [2])]
    window_switch(False)
    jp128 = gpu_adjoint(psi, obs, ops, list(range(npar)), N.PLK_C128)
    window_switch(True)
    jw = gpu_adjoint(psi, obs, ops, list(range(npar)), N.PLK_C64)
    np.testing.assert_allclose(jw, jp128, atol=1e-4, rtol=0)


def test_window_switch_roundtrip(window_switch):
    v = C.c_int32()
    window_switch(False)
    N.check(N.lib.plk_get_window_path(C.byref(v)))
    assert v.value == 0
    window_switch(True)
    N.check(N.lib.plk_get_window_path(C.byref(v)))
    assert v.value == 1



@pytest.mark.parametrize("dtype", [N.PLK_C64, N.PLK_C128])
@pytest.mark.parametrize("nobs", [2, 5])
def test_window_adjoint_several_observables(dtype, nobs, window_switch):
    """Several observables: the window program runs once per observable on
    a copy of lambda; rows match the oracle and the op-at-a-time path."""
    rng = np.random.default_rng(200 + nobs)
    nq = 10
    ops = random_circuit(nq, 90, rng)
    npar = sum(1 for o in ops if o[3])
    trainable = sorted(int(x) for x in rng.choice(npar, max(1, npar * 3 // 4), replace=False))
    obs = [("named", "PauliZ", [o % nq]) for o in range(nobs - 1)]
    obs.append(("hamiltonian", [0.5, -1.2], [("named", "PauliX", [2]),
                                             ("tensor", [("named", "PauliY", [0]), ("named", "PauliZ", [nq - 1])])]))
    psi = O.run_ops(O.zero_state(nq), ops)
    ref = O.adjoint_jacobian(psi, obs, ops, trainable)
    window_switch(True)
    jw = gpu_adjoint(psi, obs, ops, trainable, dtype)
    jw2 = gpu_adjoint(psi, obs, ops, trainable, dtype)
    window_switch(False)
    jp = gpu_adjoint(psi, obs, ops, trainable, dtype)
    np.testing.assert_array_equal(jw, jw2)
    tol = 1e-10 if dtype == N.PLK_C128 else 1e-4
    np.testing.assert_allclose(jw, ref, atol=tol, rtol=0)
    np.testing.assert_allclose(jw, jp, atol=tol, rtol=0)


def diagonal_heavy_circuit(nq, layers, rng, trainable_multi=True):
    """Layers whose diagonal ops (RZ, PhaseShift, Z, S, T, CZ, CRZ, IsingZZ,
    MultiRZ, ControlledPhaseShift) sit between rotations and CNOTs, including
    repeated RZ on one wire: the complex128 windows merge such runs."""
    ops = []
    ang = lambda: [float(rng.uniform(0, 2 * np.pi))]  # noqa: E731
    for _ in range(layers):
        for w in range(nq):
            ops.append(("RY", [w], False, ang()))
            ops.append(("RZ", [w], bool(rng.integers(2)), ang()))
            if w % 3 == 0:
                ops.append(("RZ", [w], False, ang()))
                ops.append(("PhaseShift", [w], bool(rng.integers(2)), ang()))
            if w % 4 == 1:
                ops.append((str(rng.choice(["PauliZ", "S", "T"])), [w], bool(rng.integers(2)), []))
        for w in range(nq - 1):
            ops.append(("CNOT", [w, w + 1], False, []))
            if w % 3 == 1:
                ops.append(("CZ", [w, w + 1], False, []))
        a, b = (int(x) for x in rng.choice(nq, 2, replace=False))
        ops.append(("CRZ", [a, b], False, ang()))
        ops.append(("ControlledPhaseShift", [b, a], False, ang()))
        if trainable_multi:
            ops.append(("IsingZZ", [a, (a + 1) % nq], False, ang()))
            ops.append(("MultiRZ", [int(x) for x in rng.choice(nq, 3, replace=False)], False, ang()))
    return ops


@pytest.mark.parametrize("nq", [7, 10, 13])
def test_window_c128_diagonal_runs(nq, window_switch):
    rng = np.random.default_rng(300 + nq)
    ops = diagonal_heavy_circuit(nq, 3, rng)
    window_switch(True)
    a = run_forward(nq, ops, N.PLK_C128)
    np.testing.assert_allclose(a, oracle_forward(nq, ops), atol=1e-12, rtol=0)
    npar = sum(1 for o in ops if o[3])
    trainable = sorted(int(x) for x in rng.choice(npar, npar * 3 // 4, replace=False))
    obs = [("hamiltonian", [0.9, -0.6], [("named", "PauliX", [1]),
                                         ("tensor", [("named", "PauliZ", [0]), ("named", "PauliY", [nq - 1])])])]
    psi = O.run_ops(O.zero_state(nq), ops)
    ref = O.adjoint_jacobian(psi, obs, ops, trainable)
    jw = gpu_adjoint(psi, obs, ops, trainable, N.PLK_C128)
    jw2 = gpu_adjoint(psi, obs, ops, trainable, N.PLK_C128)
    np.testing.assert_array_equal(jw, jw2)
    np.testing.assert_allclose(jw, ref, atol=1e-10, rtol=0)
