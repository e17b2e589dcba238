"""GPU parity on states whose amplitudes span thirty decades (1e-30 ... 1).

complex128 kernels compute in double-float on the FP32 pipe by default: each
double is an unevaluated sum of two floats, so the parts have the FP32
exponent range (values below about 2^-103 lose their low part, below 2^-126
they become zero).  These tests run the same gates, op lists, expectation
values and probabilities in both complex128 modes — double-float and native
FP64 (plk_set_c128_arithmetic) — on such states and compare each with the
oracle:

* states within 1e-12 elementwise (absolute), and, for gates that only
  permute amplitudes or multiply them by phases (so tiny amplitudes stay
  tiny), within 1e-12 relative for every amplitude of magnitude >= 1e-28;
* expectation values and probabilities within 1e-10.
"""
import ctypes as C
import zlib

import numpy as np
import pytest

import oracle as O
from abi import State, make_ops
from pennylane_lightning_kokkos import _native as N
from test_oracle_golden import ALL_GATES

pytestmark = pytest.mark.gpu

MODES = ["double-float", "fp64"]
# gates that only permute amplitudes or multiply them by phases
NON_MIXING = {"PauliX", "PauliY", "PauliZ", "S", "T", "PhaseShift", "RZ", "CNOT", "CY", "CZ", "SWAP",
              "ControlledPhaseShift", "CRZ", "IsingZZ", "CSWAP", "Toffoli", "MultiRZ"}


@pytest.fixture(params=MODES)
def mode(request):
    before = N.c128_arithmetic()
    N.set_c128_arithmetic(request.param)
    yield request.param
    N.set_c128_arithmetic(before)


def wide_state(nq, rng, lo_exp=-30.0):
    """Random phases, magnitudes 10^u with u uniform in [lo_exp, 0], a few
    amplitudes pinned at the extremes, normalised."""
    n = 1 << nq
    mag = 10.0 ** rng.uniform(lo_exp, 0.0, n)
    mag[rng.choice(n, 8, replace=False)] = 10.0 ** lo_exp
    mag[rng.integers(n)] = 1.0
    v = mag * np.exp(1j * rng.uniform(0, 2 * np.pi, n))
    return (v / np.linalg.norm(v)).astype(np.complex128)


def check_state(got, ref, name, relative):
    np.testing.assert_allclose(got, ref, atol=1e-12, rtol=0, err_msg=name)
    if relative:
        big = np.abs(ref) >= 1e-28
        rel = np.abs(got[big] - ref[big]) / np.abs(ref[big])
        assert rel.max() <= 1e-12, f"{name}: relative error {rel.max():.3e} on amplitudes >= 1e-28"


@pytest.mark.parametrize("name", sorted(ALL_GATES))
def test_gate_on_wide_state(name, mode):
    nw, npar = ALL_GATES[name]
    rng = np.random.default_rng(zlib.crc32(f"{name}/wide".encode()))
    nq = max(nw + 2, 8)
    for _ in range(3):
        psi = wide_state(nq, rng)
        wires = [int(w) for w in rng.choice(nq, nw, replace=False)]
        params = list(rng.uniform(0, 2 * np.pi, npar))
        inv = bool(rng.integers(2))
        ref = O.apply(psi.copy(), name, wires, inv, params)
        s = State.from_array(psi)
        s.apply(name, wires, inv, params)
        check_state(s.get(), ref, f"{name} {wires} inv={inv} ({mode})", name in NON_MIXING)
        s.close()


@pytest.mark.parametrize("k", [1, 2, 3, 4, 5])
def test_dense_matrix_on_wide_state(k, mode):
    rng = np.random.default_rng(40 + k)
    nq = 9
    z = rng.normal(size=(1 << k, 1 << k)) + 1j * rng.normal(size=(1 << k, 1 << k))
    q, r = np.linalg.qr(z)
    u = q * (np.diag(r) / np.abs(np.diag(r)))
    psi = wide_state(nq, rng)
    wires = [int(w) for w in rng.choice(nq, k, replace=False)]
    ref = O.apply_matrix(psi.copy(), u, wires)
    s = State.from_array(psi)
    s.apply_matrix(u, wires)
    check_state(s.get(), ref, f"Haar {k}q {wires} ({mode})", False)


def test_op_list_on_wide_state(mode):
    # a layered circuit through plk_apply_ops (register windows in double-float mode)
    rng = np.random.default_rng(77)
    nq = 10
    ops = []
    for layer in range(3):
        for w in range(nq):
            ops.append(("RZ", [w], False, [float(rng.uniform(0, 2 * np.pi))]))
            if layer == 2 and w % 3 == 0:
                ops.append(("RY", [w], False, [float(rng.uniform(0, 0.2))]))
        for w in range(nq - 1):
            ops.append(("CNOT", [w, w + 1], False, []))
    psi = wide_state(nq, rng)
    ref = O.run_ops(psi.copy(), ops)
    s = State.from_array(psi)
    arr, keep = make_ops(ops)
    N.check(N.lib.plk_apply_ops(s.h, arr, len(ops)))
    check_state(s.get(), ref, f"op list ({mode})", False)


def test_measurements_on_wide_state(mode):
    rng = np.random.default_rng(91)
    nq = 12
    psi = wide_state(nq, rng)
    s = State.from_array(psi)
    for name in ("PauliX", "PauliY", "PauliZ", "Hadamard", "Identity"):
        for w in (0, 5, nq - 1):
            assert abs(s.expval_named(name, [w]) - O.expval_named(psi, name, [w])) <= 1e-10, (name, w)
    for k in (1, 2, 3):
        m = rng.normal(size=(1 << k, 1 << k)) + 1j * rng.normal(size=(1 << k, 1 << k))
        wires = [int(w) for w in rng.choice(nq, k, replace=False)]
        assert abs(s.expval_matrix(m, wires) - O.expval_matrix(psi, m, wires)) <= 1e-10, (k, wires)
    np.testing.assert_allclose(s.probs(), O.probs(psi), atol=1e-10, rtol=0)
    for wires in ([3], [0, 11], [7, 2, 9]):
        np.testing.assert_allclose(s.probs(wires), O.probs(psi, wires), atol=1e-10, rtol=0, err_msg=str(wires))
    re, im = C.c_double(), C.c_double()
    t = State.from_array(wide_state(nq, rng))
    N.check(N.lib.plk_inner_product(s.h, t.h, C.byref(re), C.byref(im)))
    ref = np.vdot(psi, t.get())
    assert abs(re.value - ref.real) <= 1e-10 and abs(im.value - ref.imag) <= 1e-10
    # tiny probabilities: every bin below 1e-40 is reproduced to 1e-10 (absolute)
    p = s.probs()
    tiny = O.probs(psi) < 1e-40
    assert tiny.any() and np.all(np.abs(p[tiny]) <= 1e-10)
