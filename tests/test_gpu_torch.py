"""GPU: the torch autograd layer (adjoint backward) against finite differences
and the oracle's restatement of the reference adjoint_jacobian.

Tolerances: complex128 gradients within 1e-7 of central finite differences
(h = 1e-6, complex128 forward passes) and within 1e-10 of the oracle;
complex64 gradients (FP64-class accumulation) within 1e-5 of complex128.
"""
import numpy as np
import pytest

import oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def ansatz(nq, layers, seed):
    from pennylane_lightning_kokkos.circuits import hardware_efficient_ansatz

    ops = hardware_efficient_ansatz(nq, layers, seed, rotations=("RY", "RZ"), entangler="ladder")
    params = np.array([o[3][0] for o in ops if o[3]])
    return [(o[0], o[1]) for o in ops], params, ops


def words_to_obs(words):
    terms = []
    for c, w, l in words:
        f = [("named", {"X": "PauliX", "Y": "PauliY", "Z": "PauliZ"}[x], [wi]) for wi, x in zip(w, l)]
        terms.append(("tensor", f))
    return ("hamiltonian", [c for c, _, _ in words], terms)


def test_gradient_vs_central_differences_14q():
    from pennylane_lightning_kokkos.circuits import random_pauli_words
    from pennylane_lightning_kokkos.torch_adjoint import AdjointCircuit

    nq = 14
    struct, params, _ = ansatz(nq, 3, seed=4)
    words = random_pauli_words(nq, 20, seed=4)
    circ = AdjointCircuit(nq, struct, [words], dtype="c128")
    x = torch.tensor(params, dtype=torch.float64, requires_grad=True)
    y = circ(x)
    y.sum().backward()
    g = x.grad.numpy()
    h = 1e-6
    rng = np.random.default_rng(0)
    for i in rng.choice(len(params), 24, replace=False):
        pp, pm = params.copy(), params.copy()
        pp[i] += h
        pm[i] -= h
        fd = (circ(torch.tensor(pp)).item() - circ(torch.tensor(pm)).item()) / (2 * h)
        assert abs(g[i] - fd) < 1e-7, (i, g[i], fd)


def test_gradient_matches_oracle_adjoint():
    from pennylane_lightning_kokkos.circuits import random_pauli_words
    from pennylane_lightning_kokkos.torch_adjoint import AdjointCircuit

    nq = 8
    struct, params, ops = ansatz(nq, 4, seed=1)
    obs_words = [random_pauli_words(nq, 6, seed=s) for s in (1, 2, 3)]
    gout = np.array([0.7, -1.3, 0.25])
    psi = O.run_ops(O.zero_state(nq), ops)
    ref_vals = [O.expval_observable(psi, words_to_obs(w)) for w in obs_words]
    ref_jac = O.adjoint_jacobian(psi, [words_to_obs(w) for w in obs_words], ops, list(range(len(params))))
    for dtype, tol in (("c128", 1e-10), ("c64", 1e-4)):
        circ = AdjointCircuit(nq, struct, obs_words, dtype=dtype)
        x = torch.tensor(params, requires_grad=True)
        y = circ(x)
        np.testing.assert_allclose(y.detach().numpy(), ref_vals, atol=tol)
        y.backward(torch.tensor(gout))
        np.testing.assert_allclose(x.grad.numpy(), gout @ ref_jac, atol=tol)


def test_c64_vs_c128_and_recompute_mode():
    from pennylane_lightning_kokkos.circuits import random_pauli_words
    from pennylane_lightning_kokkos.torch_adjoint import AdjointCircuit

    nq = 12
    struct, params, _ = ansatz(nq, 5, seed=7)
    words = random_pauli_words(nq, 30, seed=7)
    grads = {}
    for dtype in ("c128", "c64"):
        for rec in (False, True):
            circ = AdjointCircuit(nq, struct, [words], dtype=dtype, recompute=rec)
            x = torch.tensor(params, requires_grad=True)
            circ(x).sum().backward()
            grads[(dtype, rec)] = x.grad.numpy().copy()
    np.testing.assert_array_equal(grads[("c128", False)], grads[("c128", True)])
    np.testing.assert_array_equal(grads[("c64", False)], grads[("c64", True)])
    assert np.max(np.abs(grads[("c64", False)] - grads[("c128", False)])) < 1e-5


def test_rot_decomposition_and_errors():
    from pennylane_lightning_kokkos.torch_adjoint import AdjointCircuit

    circ = AdjointCircuit(2, [("Rot", [0]), ("CNOT", [0, 1])], [[(1.0, [1], "Z")]], dtype="c128")
    assert circ.num_params == 3
    x = torch.tensor([0.1, 0.7, -0.4], requires_grad=True)
    circ(x).sum().backward()
    ops = [("RZ", [0], False, [0.1]), ("RY", [0], False, [0.7]), ("RZ", [0], False, [-0.4]),
           ("CNOT", [0, 1], False, [])]
    psi = O.run_ops(O.zero_state(2), ops)
    ref = O.adjoint_jacobian(psi, [("named", "PauliZ", [1])], ops, [0, 1, 2])[0]
    np.testing.assert_allclose(x.grad.numpy(), ref, atol=1e-12)
    with pytest.raises(ValueError):
        AdjointCircuit(2, [("CRot", [0, 1])], [[(1.0, [1], "Z")]])
