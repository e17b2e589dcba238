"""GPU parity: adjoint Jacobian through the C ABI and the pybind module.

Tolerances: complex128 Jacobians within 1e-10 of the oracle's restatement of
AdjointJacobianKokkos::adjointJacobian; complex64 states with FP64
inner-product accumulation within 1e-4 (absolute) of the same FP64 oracle.
"""
import ctypes as C

import numpy as np
import pytest

import known_answers as KA
import oracle as O
from abi import State, i64, make_ops
from pennylane_lightning_kokkos import _native as N
from test_oracle_golden import ALL_GATES, rand_state, state_from

pytestmark = pytest.mark.gpu

JTOL = {N.PLK_C128: 1e-10, N.PLK_C64: 1e-4}
DTYPES = [N.PLK_C128, N.PLK_C64]


def gpu_adjoint(psi_fwd, observables, ops, trainable, dtype):
    """plk_adjoint_jacobian with H|lambda> states prepared by the oracle."""
    lam = State.from_array(psi_fwd, dtype)
    hls = []
    for o in observables:
        h = O.apply_observable(psi_fwd.copy(), o)
        hls.append(State.from_array(h, dtype))
    harr = (C.c_void_p * max(1, len(hls)))(*[h.h.value for h in hls])
    arr, keep = make_ops(ops)
    tp, tpp = i64(trainable)
    jac = np.zeros((len(observables), len(trainable)))
    N.check(N.lib.plk_adjoint_jacobian(lam.h, harr, len(hls), arr, len(ops), tpp, len(trainable),
                                       jac.ctypes.data_as(C.POINTER(C.c_double))))
    return jac


@pytest.mark.parametrize("case", sorted(KA.ADJOINT_CASES))
def test_adjoint_known_answers_gpu(case):
    init, nq, ops, obs, tp, expected, margin = KA.ADJOINT_CASES[case]
    psi = O.run_ops(state_from(init, nq), ops)
    jac = gpu_adjoint(psi, obs, ops, tp, N.PLK_C128)
    for i, row in enumerate(expected):
        for j, e in enumerate(row):
            if e is not None:
                assert jac[i, j] == pytest.approx(e, abs=margin), (i, j, jac)


PARAM_GATES = [g for g, (nw, npar) in ALL_GATES.items() if npar == 1]


def random_circuit(nq, nops, rng, gates=None):
    gates = gates or sorted(ALL_GATES)
    ops = []
    for _ in range(nops):
        name = str(rng.choice(gates))
        nw, npar = ALL_GATES[name]
        if npar > 1:
            continue  # Rot/CRot are decomposed before differentiation
        ops.append((name, [int(w) for w in rng.choice(nq, nw, replace=False)], bool(rng.integers(2)),
                    list(rng.uniform(0, 2 * np.pi, npar))))
    return ops


@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("seed", [0, 1, 2])
def test_adjoint_random_circuits(seed, dtype):
    rng = np.random.default_rng(seed)
    nq = 7
    ops = random_circuit(nq, 60, rng)
    npar = sum(1 for o in ops if o[3])
    trainable = sorted(int(x) for x in rng.choice(npar, max(1, npar * 2 // 3), replace=False))
    obs = [("named", "PauliZ", [w]) for w in range(nq)]
    obs += [("tensor", [("named", "PauliX", [0]), ("named", "PauliY", [3])]),
            ("hamiltonian", [0.3, -1.2], [("named", "PauliZ", [1]), ("named", "PauliX", [5])]),
            ("hermitian", np.diag([1.0, -2.0, 0.5, 3.0]).astype(complex), [2, 6])]
    psi = O.run_ops(O.zero_state(nq), ops)
    ref = O.adjoint_jacobian(psi, obs, ops, trainable)
    jac = gpu_adjoint(psi, obs, ops, trainable, dtype)
    np.testing.assert_allclose(jac, ref, atol=JTOL[dtype], rtol=0)


@pytest.mark.parametrize("name", PARAM_GATES)
def test_adjoint_each_parametric_gate(name):
    rng = np.random.default_rng(len(name))
    nq = 6
    nw = ALL_GATES[name][0]
    ops = [("RY", [w], False, [float(rng.uniform(0, 6))]) for w in range(nq)]
    ops += [(name, [int(w) for w in rng.choice(nq, nw, replace=False)], inv, [float(rng.uniform(0, 6))])
            for inv in (False, True)]
    ops += [("CNOT", [w, w + 1], False, []) for w in range(nq - 1)]
    npar = sum(1 for o in ops if o[3])
    obs = [("named", "PauliX", [0]), ("named", "PauliZ", [nq - 1])]
    psi = O.run_ops(O.zero_state(nq), ops)
    ref = O.adjoint_jacobian(psi, obs, ops, list(range(npar)))
    for dtype in DTYPES:
        np.testing.assert_allclose(gpu_adjoint(psi, obs, ops, list(range(npar)), dtype), ref, atol=JTOL[dtype])


def test_adjoint_rejects_multi_parameter_ops():
    ops = [("Rot", [0], False, [0.1, 0.2, 0.3])]
    psi = O.run_ops(O.zero_state(2), ops)
    with pytest.raises(N.NativeError, match="not supported using the adjoint"):
        gpu_adjoint(psi, [("named", "PauliZ", [0])], ops, [0], N.PLK_C128)


# --------------------------------------------------------------------------
# through the reference-facing pybind module
# --------------------------------------------------------------------------
def test_pybind_adjoint_matches_oracle():
    import pennylane_lightning_kokkos.lightning_kokkos_qubit_ops as m

    rng = np.random.default_rng(11)
    nq = 6
    ops = random_circuit(nq, 40, rng)
    npar = sum(1 for o in ops if o[3])
    tp = list(range(npar))
    for bits, tol in (("128", 1e-10), ("64", 1e-4)):
        sv = getattr(m, "LightningKokkos_C" + bits)(nq)
        sv.apply([o[0] for o in ops], [o[1] for o in ops], [o[2] for o in ops], [o[3] for o in ops])
        Named = getattr(m, "NamedObsKokkos_C" + bits)
        Tensor = getattr(m, "TensorProdObsKokkos_C" + bits)
        Ham = getattr(m, "HamiltonianKokkos_C" + bits)
        Herm = getattr(m, "HermitianObsKokkos_C" + bits)
        dt = np.float64 if bits == "128" else np.float32
        cdt = np.complex128 if bits == "128" else np.complex64
        hmat = np.diag([1.0, -1.0, 2.0, 0.5]).astype(cdt)
        obs = [Named("PauliZ", [0]), Tensor([Named("PauliX", [1]), Named("PauliY", [4])]),
               Ham(np.array([0.4, -0.9], dtype=dt), [Named("PauliZ", [2]), Tensor([Named("PauliX", [3]),
                                                                                   Named("PauliZ", [5])])]),
               Herm(hmat, [1, 3])]
        adj = getattr(m, "AdjointJacobianKokkos_C" + bits)()
        ops_struct = adj.create_ops_list([o[0] for o in ops], [np.array(o[3], dtype=dt) for o in ops],
                                         [o[1] for o in ops], [o[2] for o in ops], [np.array([], dtype=cdt)] * len(ops))
        jac = adj.adjoint_jacobian(sv, obs, ops_struct, tp)
        oobs = [("named", "PauliZ", [0]), ("tensor", [("named", "PauliX", [1]), ("named", "PauliY", [4])]),
                ("hamiltonian", [0.4, -0.9], [("named", "PauliZ", [2]),
                                              ("tensor", [("named", "PauliX", [3]), ("named", "PauliZ", [5])])]),
                ("hermitian", hmat.astype(complex), [1, 3])]
        psi = O.run_ops(O.zero_state(nq), ops)
        ref = O.adjoint_jacobian(psi, oobs, ops, tp)
        np.testing.assert_allclose(jac, ref, atol=tol)


def test_pybind_known_answers():
    """Reference C++ unit-test values through the Python module."""
    import pennylane_lightning_kokkos.lightning_kokkos_qubit_ops as m

    sv = m.LightningKokkos_C128(np.array(KA.INI_3Q_C, dtype=np.complex128))
    assert sv.ExpectationValue([0, 1, 2], np.array(KA.HERMITIAN_3Q_MATRIX, dtype=np.complex128)) == pytest.approx(
        KA.EXPVAL_HERMITIAN_3Q, rel=1e-7)
    assert sv.ExpectationValue(np.array(KA.SPARSE_VALUES, dtype=np.complex128), KA.SPARSE_INDICES,
                               KA.SPARSE_INDPTR) == pytest.approx(KA.EXPVAL_SPARSE, rel=1e-7)
    sv3 = m.LightningKokkos_C128(3)
    for name, w, inv, p in KA.PROBS_INIT_OPS:
        getattr(sv3, name)(w, inv, p)
    for wires, exp in KA.PROBS_CASES:
        np.testing.assert_allclose(sv3.probs(wires), exp, atol=KA.PROBS_MARGIN)
    s = sv3.GenerateSamples(3, 1000)
    assert s.shape == (1000, 3) and s.dtype == np.uintp
    out = np.zeros(8, dtype=np.complex128)
    sv3.DeviceToHost(out)
    assert abs(np.linalg.norm(out) - 1) < 1e-12
    # gate known answers
    for case, (init, nq, ops, expected, tol) in KA.GATE_CASES.items():
        st = m.LightningKokkos_C128(nq) if init is None else m.LightningKokkos_C128(np.array(init, complex))
        for name, w, inv, p in ops:
            getattr(st, name)(w, inv, p)
        got = np.zeros(1 << nq, dtype=np.complex128)
        st.DeviceToHost(got)
        np.testing.assert_allclose(got, expected, rtol=tol, atol=tol, err_msg=case)
    with pytest.raises(m.PLException):
        sv3.RX([5], False, [0.1])


@pytest.mark.parametrize("bits", ["64", "128"])
def test_pybind_queued_copies_two_streams(bits):
    """HostToDeviceAsync / DeviceToHostAsync on two states with their own
    streams, interleaved with gates: each state ends as the oracle's."""
    import torch

    import pennylane_lightning_kokkos.lightning_kokkos_qubit_ops as m

    cls = getattr(m, "LightningKokkos_C" + bits)
    cdt = np.complex128 if bits == "128" else np.complex64
    tol = 1e-12 if bits == "128" else 1e-5
    nq = 12
    rng = np.random.default_rng(41)
    streams = [torch.cuda.Stream(), torch.cuda.Stream()]
    svs = [cls(nq), cls(nq)]
    ins, outs, refs = [], [], []
    for k in range(2):
        svs[k].set_stream(streams[k].cuda_stream)
        psi = rand_state(nq, rng)
        ins.append(torch.from_numpy(psi.astype(cdt)).pin_memory().numpy())
        outs.append(torch.zeros(1 << nq, dtype=torch.complex128 if bits == "128" else torch.complex64).pin_memory()
                    .numpy())
        ops = [("RX", [k + 1], False, [0.3 + k]), ("CNOT", [k, 7], False, []), ("IsingXX", [2, 9], False, [0.7])]
        refs.append((psi, ops))
    for k in range(2):
        svs[k].HostToDeviceAsync(ins[k])
    for k in range(2):
        for name, w, inv, p in refs[k][1]:
            getattr(svs[k], name)(w, inv, p)
        svs[k].DeviceToHostAsync(outs[k])
    for k in range(2):
        svs[k].synchronize()
        ref = O.run_ops(refs[k][0].astype(cdt).astype(np.complex128), refs[k][1])
        np.testing.assert_allclose(outs[k], ref, atol=tol)
    with pytest.raises(TypeError):  # no silent conversion copy for a queued copy
        svs[0].HostToDeviceAsync(np.zeros(1 << nq, dtype=np.complex64 if bits == "128" else np.complex128))
