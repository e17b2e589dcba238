"""GPU: batched circuits (plk_batch_*) against the oracle.

Every circuit of a batch must give the oracle's expectation value and adjoint
Jacobian (oracle.adjoint_jacobian restates AdjointDiffKokkos.hpp:404-478):
complex128 within 1e-10, complex64 (FP64-class accumulation) within 1e-4.
The engine's placements (shared memory, global memory on one CTA, global
memory shared by a cluster of 2, 4 or 8 CTAs) must all agree.
"""
import zlib

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

ONE_PARAM = {"RX": 1, "RY": 1, "RZ": 1, "PhaseShift": 1, "CRX": 2, "CRY": 2, "CRZ": 2, "ControlledPhaseShift": 2,
             "IsingXX": 2, "IsingXY": 2, "IsingYY": 2, "IsingZZ": 2, "SingleExcitation": 2,
             "SingleExcitationMinus": 2, "SingleExcitationPlus": 2, "DoubleExcitation": 4,
             "DoubleExcitationMinus": 4, "DoubleExcitationPlus": 4, "MultiRZ": 0}
FIXED = {"PauliX": 1, "PauliY": 1, "PauliZ": 1, "Hadamard": 1, "S": 1, "T": 1, "CNOT": 2, "CY": 2, "CZ": 2,
         "SWAP": 2, "CSWAP": 3, "Toffoli": 3, "Identity": 1}


def rng_for(*key):
    return np.random.default_rng(zlib.crc32(repr(key).encode()))


def random_ops(rng, nq, nops, fixed_frac=0.4):
    ops = []
    names1, names0 = list(ONE_PARAM), list(FIXED)
    for _ in range(nops):
        if rng.random() < fixed_frac:
            name = names0[rng.integers(len(names0))]
            k = FIXED[name]
            prm = []
        else:
            name = names1[rng.integers(len(names1))]
            k = ONE_PARAM[name] or int(rng.integers(1, min(nq, 6) + 1))
            prm = [float(rng.uniform(-np.pi, np.pi))]
        if k > nq:
            continue
        wires = [int(w) for w in rng.choice(nq, size=k, replace=False)]
        ops.append((name, wires, bool(rng.random() < 0.3), prm))
    return ops


def random_words(rng, nq, nterms):
    words = []
    for _ in range(nterms):
        k = int(rng.integers(1, min(4, nq) + 1))
        w = [int(x) for x in rng.choice(nq, size=k, replace=False)]
        words.append((float(rng.normal()), w, "".join(rng.choice(list("XYZ"), size=k))))
    return words


def words_to_obs(words):
    letters = {"X": "PauliX", "Y": "PauliY", "Z": "PauliZ"}
    terms = [("tensor", [("named", letters[x], [wi]) for wi, x in zip(w, l)]) for _, w, l in words]
    return ("hamiltonian", [c for c, _, _ in words], terms)


def oracle_ref(nq, ops, words, trainable):
    psi = O.run_ops(O.zero_state(nq), ops)
    obs = words_to_obs(words)
    ev = O.expval_observable(psi, obs)
    jac = O.adjoint_jacobian(psi, [obs], ops, trainable)[0] if len(trainable) else np.zeros(0)
    return ev, jac


def make_cases(tag, sizes, nops, seed_base=0):
    cases = []
    for i, nq in enumerate(sizes):
        rng = rng_for(tag, i, seed_base)
        ops = random_ops(rng, nq, nops)
        npar = sum(1 for o in ops if o[3])
        tp = sorted(int(t) for t in rng.choice(npar, size=max(1, npar * 2 // 3), replace=False)) if npar else []
        words = random_words(rng, nq, int(rng.integers(1, 8)))
        cases.append((nq, ops, words, tp))
    return cases


def run_batch(cases, dtype, config=None, graph=True):
    from pennylane_lightning_kokkos.batch import CircuitBatch

    b = CircuitBatch(dtype)
    for nq, ops, words, tp in cases:
        b.add(nq, ops, words, tp)
    if config:
        b.set_config(**config)
    b.set_graph(graph)
    ev, jac = b.run()
    grads = b.gradients(jac)
    b.close()
    return ev, grads


def check_against_oracle(cases, ev, grads, tol):
    for (nq, ops, words, tp), e, g in zip(cases, ev, grads):
        ref_e, ref_j = oracle_ref(nq, ops, words, tp)
        assert abs(e - ref_e) < tol, (nq, e, ref_e)
        np.testing.assert_allclose(g, ref_j, atol=tol, rtol=0)


SMALL = make_cases("small", [4, 5, 6, 7, 8, 9, 10, 5, 6, 7, 8, 4], 40)


def test_batch_all_gates_c128_shared_memory():
    ev, grads = run_batch(SMALL, "c128")
    check_against_oracle(SMALL, ev, grads, 1e-10)


def test_batch_all_gates_c64():
    ev, grads = run_batch(SMALL, "c64")
    check_against_oracle(SMALL, ev, grads, 1e-4)


@pytest.mark.parametrize("config", [
    dict(cluster=1, smem_qubits=4, cluster_min_qubits=30),   # every circuit in global memory, one CTA
    dict(cluster=2, smem_qubits=5, cluster_min_qubits=6),
    dict(cluster=4, smem_qubits=6, cluster_min_qubits=7),
    dict(cluster=8, smem_qubits=4, cluster_min_qubits=5),
])
def test_batch_placements_c128(config):
    ev, grads = run_batch(SMALL, "c128", config)
    check_against_oracle(SMALL, ev, grads, 1e-10)


def test_batch_two_ctas_per_sm_c64():
    cases = SMALL + make_cases("two", [13, 14, 11], 40)
    for cfg in (dict(cluster=1, ctas_per_sm=2), dict(cluster=4, ctas_per_sm=2, cluster_min_qubits=13)):
        ev, grads = run_batch(cases, "c64", cfg)
        check_against_oracle(cases, ev, grads, 1e-4)


def test_batch_larger_circuits_clusters():
    cases = make_cases("large", [13, 14, 15, 16, 12, 14], 60)
    for dtype, tol, sq in (("c128", 1e-10, 12), ("c64", 1e-4, 13)):
        ev, grads = run_batch(cases, dtype, dict(cluster=4, smem_qubits=sq, cluster_min_qubits=14))
        check_against_oracle(cases, ev, grads, tol)


def test_batch_reproducible_and_graph():
    a = run_batch(SMALL, "c64", graph=True)
    b = run_batch(SMALL, "c64", graph=True)
    c = run_batch(SMALL, "c64", graph=False)
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[0], c[0])
    for x, y, z in zip(a[1], b[1], c[1]):
        np.testing.assert_array_equal(x, y)
        np.testing.assert_array_equal(x, z)


def test_batch_set_params_and_rerun():
    from pennylane_lightning_kokkos.batch import CircuitBatch

    cases = SMALL[:6]
    b = CircuitBatch("c128")
    for nq, ops, words, tp in cases:
        b.add(nq, ops, words, tp)
    b.run()
    rng = rng_for("params")
    _, npar, _ = b.info()
    newp = rng.uniform(-np.pi, np.pi, size=npar)
    ev, jac = b.run(newp)
    grads = b.gradients(jac)
    new_cases = []
    k = 0
    for nq, ops, words, tp in cases:
        nops = []
        for name, w, inv, p in ops:
            if p:
                nops.append((name, w, inv, [float(newp[k])]))
                k += 1
            else:
                nops.append((name, w, inv, p))
        new_cases.append((nq, nops, words, tp))
    check_against_oracle(new_cases, ev, grads, 1e-10)
    b.close()


def test_batch_rot_and_matrices_vs_oracle():
    """Rot / CRot are decomposed (all three angles differentiable); matrix ops
    (1-4 wires, inverse = conjugate transpose) take part in the forward pass."""
    from pennylane_lightning_kokkos.batch import CircuitBatch
    from pennylane_lightning_kokkos.circuits import haar_unitary

    rng = rng_for("rotmat")
    nq = 6
    cases = []
    for i in range(4):
        ops, ref_ops = [], []
        for k in range(30):
            r = rng.random()
            if r < 0.3:
                name = "Rot" if rng.random() < 0.5 else "CRot"
                w = [int(x) for x in rng.choice(nq, size=1 if name == "Rot" else 2, replace=False)]
                p = [float(x) for x in rng.uniform(-np.pi, np.pi, 3)]
                inv = bool(rng.random() < 0.3)
                ops.append((name, w, inv, p))
                z, y = ("RZ", "RY") if name == "Rot" else ("CRZ", "CRY")
                seq = [(z, p[0]), (y, p[1]), (z, p[2])]
                if inv:
                    seq = seq[::-1]
                ref_ops += [(g, w, inv, [a]) for g, a in seq]
            elif r < 0.5:
                kq = int(rng.integers(1, 5))
                w = [int(x) for x in rng.choice(nq, size=kq, replace=False)]
                U = haar_unitary(1 << kq, rng)
                inv = bool(rng.random() < 0.5)
                ops.append(("Matrix", w, inv, [], U))
                ref_ops.append(("Matrix", w, inv, U))
            else:
                o = random_ops(rng, nq, 1, fixed_frac=0.2)
                ops += o
                ref_ops += o
        words = random_words(rng, nq, 5)
        cases.append((ops, ref_ops, words))
    for dtype, tol in (("c128", 1e-10), ("c64", 1e-4)):
        b = CircuitBatch(dtype)
        for ops, _, words in cases:
            b.add(nq, ops, words)
        ev, jac = b.run()
        grads = b.gradients(jac)
        for (ops, ref_ops, words), e, g in zip(cases, ev, grads):
            psi = O.zero_state(nq)
            for op in ref_ops:
                if op[0] == "Matrix":
                    O.apply_matrix(psi, op[3], op[1], op[2])
                else:
                    O.apply(psi, op[0], op[1], op[2], op[3])
            ref_e = O.expval_observable(psi, words_to_obs(words))
            assert abs(e - ref_e) < tol
            # gradient: central differences of the oracle forward pass
            if dtype == "c128":
                flat = [a for op in ops if op[0] != "Matrix" for a in op[3]]
                assert len(g) == len(flat)
                for t in rng.choice(len(flat), size=min(6, len(flat)), replace=False):
                    vals = []
                    for s in (+1, -1):
                        k = 0
                        psi = O.zero_state(nq)
                        for op in ops:
                            if op[0] == "Matrix":
                                O.apply_matrix(psi, op[4], op[1], op[2])
                                continue
                            p = list(op[3])
                            for j in range(len(p)):
                                if k == t:
                                    p[j] += s * 1e-6
                                k += 1
                            O.apply(psi, op[0], op[1], op[2], p)
                        vals.append(O.expval_observable(psi, words_to_obs(words)))
                    assert abs(g[t] - (vals[0] - vals[1]) / 2e-6) < 1e-6
        b.close()


def test_batch_tune_keeps_results():
    from pennylane_lightning_kokkos.batch import CircuitBatch

    cases = make_cases("tune", [8, 12, 14, 15, 9, 16, 10, 13], 50)
    b = CircuitBatch("c64")
    for nq, ops, words, tp in cases:
        b.add(nq, ops, words, tp)
    report = b.tune(reps=2)
    assert "ms" in report
    ev, jac = b.run()
    check_against_oracle(cases, ev, b.gradients(jac), 1e-4)
    b.close()


def test_batch_errors():
    from pennylane_lightning_kokkos import _native as N
    from pennylane_lightning_kokkos.batch import CircuitBatch
    from pennylane_lightning_kokkos.circuits import haar_unitary

    b = CircuitBatch("c64")
    with pytest.raises(N.NativeError, match="wire out of range"):
        b.add(5, [("RX", [5], False, [0.1])], [(1.0, [0], "Z")])
    with pytest.raises(N.NativeError, match="at most 4 wires"):
        b.add(6, [("Matrix", [0, 1, 2, 3, 4], False, [], haar_unitary(32, np.random.default_rng(0)))],
              [(1.0, [0], "Z")])
    with pytest.raises(N.NativeError, match="trainable index out of range"):
        b.add(5, [("RX", [0], False, [0.1])], [(1.0, [0], "Z")], trainable=[1])
    with pytest.raises(N.NativeError, match="4 to 30 qubits"):
        b.add(3, [("RX", [0], False, [0.1])], [(1.0, [0], "Z")])
    with pytest.raises(N.NativeError, match="empty batch"):
        b.run()
    with pytest.raises(N.NativeError, match="Pauli letter"):
        b.add(5, [("RX", [0], False, [0.1])], [(1.0, [0], "Q")])
    b.close()


def test_batch_shards_match_one_batch():
    """A batch split by shard_plan into three shards, each run as its own
    CircuitBatch (as three GPUs would), gives the results of one batch."""
    from pennylane_lightning_kokkos.batch import CircuitBatch, run_shard, shard_plan
    from pennylane_lightning_kokkos.circuits import batch_workload_packed

    wl = batch_workload_packed(24, seed=11, min_qubits=4, max_qubits=9, min_layers=1, max_layers=4)
    costs = [len(pk["gates"]) * float(1 << nq) for nq, pk, _ in wl]
    b = CircuitBatch("c128")
    for nq, pk, words in wl:
        b.add_packed(nq, pk, words)
    ev, jac = b.run()
    grads = b.gradients(jac)
    b.close()
    shards = shard_plan(costs, 3)
    for shard in shards:
        ev_s, g_s = run_shard(wl, shard, "c128")
        for k, i in enumerate(shard):
            assert abs(ev_s[k] - ev[i]) < 1e-12
            np.testing.assert_allclose(g_s[k], grads[i], atol=1e-12, rtol=0)
