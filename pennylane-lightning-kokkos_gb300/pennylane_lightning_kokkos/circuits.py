"""Seeded synthetic circuits and Hamiltonians.

Used by the benchmark and the tests; all randomness comes from
``numpy.random.default_rng(seed)`` so a (seed, size) pair always gives the
same circuit.  Wire 0 is the most significant bit of the amplitude index.
"""
from __future__ import annotations

import numpy as np

# name -> (number of wires, fraction of the amplitudes read and written)
SWEEP_GATES = {
    "PauliX": (1, 1.0),
    "Hadamard": (1, 1.0),
    "RX": (1, 1.0),
    "CNOT": (2, 0.5),
    "CRY": (2, 0.5),
    "IsingXX": (2, 1.0),
    "SingleExcitation": (2, 0.5),
    "DoubleExcitation": (4, 0.125),
    "Haar2q": (2, 1.0),
}
PARAMETRIC = {"RX", "CRY", "IsingXX", "SingleExcitation", "DoubleExcitation"}


def haar_unitary(dim: int, rng: np.random.Generator) -> np.ndarray:
    """Haar-random unitary: QR of a complex Gaussian matrix with the phases
    of R's diagonal moved into Q (Mezzadri, Notices AMS 54 (2007) 592)."""
    z = (rng.standard_normal((dim, dim)) + 1j * rng.standard_normal((dim, dim))) / np.sqrt(2.0)
    q, r = np.linalg.qr(z)
    d = np.diag(r)
    return q * (d / np.abs(d))


def wire_ranges(nq: int) -> dict:
    """Low / mid / high wire ranges of the gate sweep.  At 30 qubits these are
    wires 0-4 (bit positions 25-29, the largest strides), 12-17 and 25-29
    (bit positions 0-4, inside one 32-amplitude run)."""
    mid0 = 12 if nq == 30 else max(0, nq // 2 - 3)
    return {"low": list(range(0, min(5, nq))), "mid": list(range(mid0, min(nq, mid0 + 6))),
            "high": list(range(max(0, nq - 5), nq))}


def gate_sweep_plan(nq: int = 30, reps: int = 4, seed: int = 2, gates=None, ranges=None):
    """Applications of the gate-throughput sweep: for every gate, every wire
    range and `reps` repetitions, distinct wires drawn uniformly inside the
    range and an angle uniform in [0, 2*pi).  Returns a list of dicts with
    name, wires, params, matrix (Haar2q only), range, touched."""
    rng = np.random.default_rng(seed)
    gates = gates or list(SWEEP_GATES)
    wr = wire_ranges(nq)
    ranges = ranges or list(wr)
    plan = []
    for g in gates:
        nw, touched = SWEEP_GATES[g]
        for rname in ranges:
            pool = wr[rname]
            for _ in range(reps):
                wires = [int(w) for w in rng.choice(pool, nw, replace=False)]
                params = [float(rng.uniform(0, 2 * np.pi))] if g in PARAMETRIC else []
                mat = haar_unitary(4, rng) if g == "Haar2q" else None
                plan.append({"name": g, "wires": wires, "params": params, "matrix": mat, "range": rname,
                             "touched": touched})
    return plan


def hardware_efficient_ansatz(nq: int, layers: int, seed: int, rotations=("RY", "RZ"), entangler: str = "ladder"):
    """Layers of single-qubit rotations on every wire followed by a CNOT
    ladder (i -> i+1, i < n-1) or ring (i -> i+1 mod n); angles uniform in
    [0, 2*pi).  Returns [(name, wires, inverse, params)]."""
    rng = np.random.default_rng(seed)
    ops = []
    for _ in range(layers):
        for w in range(nq):
            for r in rotations:
                ops.append((r, [w], False, [float(rng.uniform(0, 2 * np.pi))]))
        pairs = [(w, w + 1) for w in range(nq - 1)]
        if entangler == "ring":
            pairs = [(w, (w + 1) % nq) for w in range(nq)]
        for a, b in pairs:
            ops.append(("CNOT", [a, b], False, []))
    return ops


def random_pauli_words(nq: int, count: int, seed: int, max_weight: int = 4):
    """`count` Pauli words: weight uniform in 1..max_weight on distinct
    uniform wires, letters uniform over X/Y/Z, coefficients N(0, 1).
    Returns [(coeff, wires, letters)]."""
    rng = np.random.default_rng(seed)
    words = []
    for _ in range(count):
        wt = int(rng.integers(1, max_weight + 1))
        wires = [int(w) for w in rng.choice(nq, wt, replace=False)]
        letters = "".join(str(x) for x in rng.choice(["X", "Y", "Z"], wt))
        words.append((float(rng.standard_normal()), wires, letters))
    return words


def layered_ansatz_arrays(nq: int, angles: np.ndarray, rotations=("RX", "RY", "RZ")):
    """Packed form of hardware_efficient_ansatz with a CNOT ladder: angles has
    shape (layers, nq, len(rotations)).  Returns a dict of flat arrays (gate
    ids, wires with offsets, inverse flags, parameters with offsets)."""
    from ._native import GATE_ID

    layers, nr = angles.shape[0], len(rotations)
    per_layer = nq * nr + (nq - 1)
    rot_ids = np.array([GATE_ID[r] for r in rotations], dtype=np.int32)
    gates = np.empty((layers, per_layer), dtype=np.int32)
    gates[:, :nq * nr] = np.tile(rot_ids, nq)
    gates[:, nq * nr:] = GATE_ID["CNOT"]
    nw = np.ones((layers, per_layer), dtype=np.int64)
    nw[:, nq * nr:] = 2
    rot_w = np.repeat(np.arange(nq), nr)
    cn_w = np.stack([np.arange(nq - 1), np.arange(1, nq)], axis=1).reshape(-1)
    wires = np.tile(np.concatenate([rot_w, cn_w]), layers).astype(np.int64)
    npar = np.zeros((layers, per_layer), dtype=np.int64)
    npar[:, :nq * nr] = 1
    return {"gates": gates.reshape(-1), "wire_offsets": np.concatenate([[0], np.cumsum(nw)]).astype(np.int64),
            "wires": wires, "inverse": np.zeros(gates.size, dtype=np.int32),
            "param_offsets": np.concatenate([[0], np.cumsum(npar)]).astype(np.int64),
            "params": np.ascontiguousarray(angles, dtype=np.float64).reshape(-1)}


def packed_to_ops(pk):
    """[(name, wires, inverse, params)] from the packed form."""
    from ._native import GATES

    g, wo, w, inv, po, p = (pk["gates"], pk["wire_offsets"], pk["wires"], pk["inverse"], pk["param_offsets"],
                            pk["params"])
    return [(GATES[g[i]], [int(x) for x in w[wo[i]:wo[i + 1]]], bool(inv[i]), [float(x) for x in p[po[i]:po[i + 1]]])
            for i in range(len(g))]


def batch_workload_packed(num_circuits: int = 4096, seed: int = 5, min_qubits: int = 8, max_qubits: int = 20,
                          min_layers: int = 5, max_layers: int = 30, terms: int = 10):
    """Independent circuits of uneven size: qubits uniform in [min_qubits,
    max_qubits], depth uniform in [min_layers, max_layers] layers of RX, RY,
    RZ on every wire plus a CNOT ladder, angles uniform in [0, 2*pi), and a
    `terms`-word Pauli Hamiltonian per circuit (weight uniform in 1..4,
    distinct uniform wires, letters uniform in X/Y/Z, N(0, 1) coefficients).
    Returns [(num_qubits, packed ops, words)]."""
    rng = np.random.default_rng(seed)
    nqs = rng.integers(min_qubits, max_qubits + 1, size=num_circuits)
    depths = rng.integers(min_layers, max_layers + 1, size=num_circuits)
    out = []
    for nq, d in zip(nqs, depths):
        nq, d = int(nq), int(d)
        angles = rng.uniform(0, 2 * np.pi, size=(d, nq, 3))
        words = []
        for _ in range(terms):
            k = int(rng.integers(1, min(4, nq) + 1))
            w = [int(x) for x in rng.choice(nq, size=k, replace=False)]
            words.append((float(rng.normal()), w, "".join(rng.choice(list("XYZ"), size=k))))
        out.append((nq, layered_ansatz_arrays(nq, angles), words))
    return out


def batch_workload(num_circuits: int = 4096, seed: int = 5, **kw):
    """batch_workload_packed as [(num_qubits, ops, words)] op lists."""
    return [(nq, packed_to_ops(pk), words) for nq, pk, words in batch_workload_packed(num_circuits, seed, **kw)]
