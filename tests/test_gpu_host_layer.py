"""GPU parity of the plugin-facing measurement surface against the oracle.

* The four ``ExpectationValue`` overloads of ``LightningKokkos_C{64,128}``
  (bindings/Bindings.cpp:434-520 of the reference): by name, by a list of
  names with a matrix (the route the Python device uses for tensor
  observables and for ``var``, lightning_kokkos.py:432-456), by wires and a
  matrix, and by a CSR matrix.
* ``var`` the way the Python device computes it: <M> and <M^dag M> through the
  names-list overload, var = <M^dag M> - <M>^2.
* The C++ host layer's ``MeasuresGB::expval`` / ``MeasuresGB::var``
  (MeasuresKokkos.hpp:354-381) with Named, Tensor, Hermitian and Hamiltonian
  observables, through a small C++ driver (tests/cpp/host_measures.cpp)
  built here against libplk_gb300.so.

Tolerances: complex128 1e-10; complex64 1e-5 (expectation values) and 5e-5
(variances, which square the single-precision rounding of <M>).
"""
import os
import subprocess
import tempfile

import numpy as np
import pytest

import oracle as O
import pennylane_lightning_kokkos.lightning_kokkos_qubit_ops as m
from conftest import ROOT
from pennylane_lightning_kokkos import _native as N
from test_oracle_golden import rand_state

pytestmark = pytest.mark.gpu

BITS = ["128", "64"]
ETOL = {"128": 1e-10, "64": 1e-5}
VTOL = {"128": 1e-10, "64": 5e-5}
PAULI = {
    "PauliX": np.array([[0, 1], [1, 0]], dtype=np.complex128),
    "PauliY": np.array([[0, -1j], [1j, 0]], dtype=np.complex128),
    "PauliZ": np.array([[1, 0], [0, -1]], dtype=np.complex128),
    "Hadamard": np.array([[1, 1], [1, -1]], dtype=np.complex128) / np.sqrt(2),
}


def sv_of(bits, psi):
    cdt = np.complex128 if bits == "128" else np.complex64
    return getattr(m, "LightningKokkos_C" + bits)(np.ascontiguousarray(psi, dtype=cdt))


def cmat(bits, a):
    return np.ascontiguousarray(a, dtype=np.complex128 if bits == "128" else np.complex64)


def hermitian(k, rng):
    a = rng.normal(size=(1 << k, 1 << k)) + 1j * rng.normal(size=(1 << k, 1 << k))
    return (a + a.conj().T) / 2


@pytest.mark.parametrize("bits", BITS)
def test_expectation_value_by_name(bits):
    rng = np.random.default_rng(3)
    nq = 7
    psi = rand_state(nq, rng)
    sv = sv_of(bits, psi)
    empty = cmat(bits, [])
    for name in ("Identity", "PauliX", "PauliY", "PauliZ", "Hadamard"):
        for w in (0, 3, 6):
            got = sv.ExpectationValue(name, [w], [], empty)
            assert abs(got - O.expval_named(psi, name, [w])) < ETOL[bits], (name, w)
    # a name without a kernel takes the matrix (k = 1..4)
    for k in (1, 2, 3, 4):
        h = hermitian(k, rng)
        wires = [int(x) for x in rng.choice(nq, k, replace=False)]
        got = sv.ExpectationValue("Hermitian", wires, [], cmat(bits, h.ravel()))
        assert abs(got - O.expval_matrix(psi, h, wires)) < ETOL[bits] * 10, (k, wires)


@pytest.mark.parametrize("bits", BITS)
def test_expectation_value_names_list_and_var(bits):
    # the Python device's tensor-observable and var route (lightning_kokkos.py:432-456)
    rng = np.random.default_rng(4)
    nq = 8
    psi = rand_state(nq, rng)
    sv = sv_of(bits, psi)
    cases = [(["PauliX", "PauliZ"], [1, 5]), (["PauliY"], [6]), (["Hadamard", "PauliY", "PauliX"], [0, 7, 3])]
    for names, wires in cases:
        mat = PAULI[names[0]]
        for nm in names[1:]:
            mat = np.kron(mat, PAULI[nm])
        obs = ("tensor", [("named", nm, [w]) for nm, w in zip(names, wires)])
        mean = sv.ExpectationValue([f"{n}_var" for n in names], wires, [[] for _ in names], cmat(bits, mat.ravel()))
        sqr = mat.conj().T @ mat
        sq = sv.ExpectationValue([f"{n}_sqr" for n in names], wires, [[] for _ in names], cmat(bits, sqr.ravel()))
        assert abs(mean - O.expval_observable(psi, obs)) < ETOL[bits], names
        assert abs((sq - mean ** 2) - O.var_observable(psi, obs)) < VTOL[bits], names
    # a Hermitian tensor factor
    h = hermitian(2, rng)
    mean = sv.ExpectationValue(["Hermitian"], [2, 4], [[]], cmat(bits, h.ravel()))
    assert abs(mean - O.expval_matrix(psi, h, [2, 4])) < ETOL[bits] * 10


@pytest.mark.parametrize("bits", BITS)
def test_expectation_value_matrix_and_sparse(bits):
    rng = np.random.default_rng(5)
    nq = 6
    psi = rand_state(nq, rng)
    sv = sv_of(bits, psi)
    for k in (1, 2, 3):
        h = hermitian(k, rng)
        wires = [int(x) for x in rng.choice(nq, k, replace=False)]
        got = sv.ExpectationValue(wires, cmat(bits, h.ravel()))
        assert abs(got - O.expval_matrix(psi, h, wires)) < ETOL[bits] * 10, (k, wires)
    # a random sparse Hermitian matrix over the whole state, CSR
    dim = 1 << nq
    dense = np.zeros((dim, dim), dtype=np.complex128)
    for _ in range(3 * dim):
        r, c = rng.integers(dim, size=2)
        v = rng.normal() + 1j * rng.normal()
        dense[r, c] += v
        dense[c, r] += np.conj(v)
    rows, cols = np.nonzero(dense)
    indptr = np.searchsorted(rows, np.arange(dim + 1)).astype(np.int64)
    data = dense[rows, cols]
    got = sv.ExpectationValue(cmat(bits, data), cols.astype(np.int64), indptr)
    ref = O.expval_sparse(psi, data, cols, indptr)
    assert abs(got - ref) < ETOL[bits] * 100 * max(1.0, abs(ref))


@pytest.fixture(scope="module")
def host_driver():
    src = os.path.join(ROOT, "tests", "cpp", "host_measures.cpp")
    pkg = os.path.dirname(N.LIB_PATH)
    out = os.path.join(tempfile.mkdtemp(prefix="plk_host_"), "host_measures")
    subprocess.run([os.environ.get("CXX", "g++"), "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
                    "-I", os.path.join(ROOT, "pennylane-lightning-kokkos_gb300", "csrc"), src, "-o", out,
                    "-L", pkg, "-l:libplk_gb300.so", "-Wl,-rpath," + pkg], check=True, capture_output=True)
    return out


@pytest.mark.parametrize("bits", BITS)
def test_host_layer_expval_and_var(host_driver, bits):
    rng = np.random.default_rng(6)
    nq = 9
    psi = rand_state(nq, rng)
    h = hermitian(2, rng)
    with tempfile.TemporaryDirectory() as d:
        sp, hp = os.path.join(d, "s.bin"), os.path.join(d, "h.bin")
        psi.astype(np.complex128).tofile(sp)
        h.astype(np.complex128).tofile(hp)
        r = subprocess.run([host_driver, bits, sp, hp], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    got = {ln.split()[0]: (float(ln.split()[1]), float(ln.split()[2])) for ln in r.stdout.strip().splitlines()}
    x1, z0, y2 = ("named", "PauliX", [1]), ("named", "PauliZ", [0]), ("named", "PauliY", [2])
    zy = ("tensor", [z0, y2])
    he = ("hermitian", h, [3, 1])
    refs = {"x1": x1, "h4": ("named", "Hadamard", [4]), "zy": zy, "herm": he,
            "ham": ("hamiltonian", [0.7, -1.3, 0.4], [x1, zy, he])}
    for label, obs in refs.items():
        ev, var = got[label]
        assert abs(ev - O.expval_observable(psi, obs)) < ETOL[bits] * 10, label
        assert abs(var - O.var_observable(psi, obs)) < VTOL[bits] * 10, label
