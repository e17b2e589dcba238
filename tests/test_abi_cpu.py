"""C ABI and module surface checks that need no GPU.

* every function declared in include/plk_gb300.h is exported by
  libplk_gb300.so (and nothing undeclared with the plk_ prefix);
* the gate table agrees with the header's enum;
* the pybind11 module exposes the reference module's classes and methods
  (bindings/Bindings.cpp of the reference);
* without a device, calls fail loudly (PLException / NO_DEVICE), never fall
  back to a CPU path.
"""
import ctypes as C
import os
import re
import subprocess

import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "plk_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"PLK_API\s+[\w\s\*]+?\b(plk_\w+)\s*\(", text)))


def test_header_declares_functions():
    fns = declared_functions()
    assert len(fns) >= 40
    assert "plk_adjoint_jacobian" in fns and "plk_apply_gate" in fns


def test_library_exports_every_declared_symbol():
    from pennylane_lightning_kokkos import _native as N

    out = subprocess.run(["nm", "-D", "--defined-only", N.LIB_PATH], capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\bT (plk_\w+)", out))
    declared = set(declared_functions())
    assert declared <= exported, f"missing exports: {sorted(declared - exported)}"
    assert exported <= declared, f"undeclared exports: {sorted(exported - declared)}"
    for f in declared:
        assert hasattr(N.lib, f)


def test_gate_table_matches_header_enum():
    from pennylane_lightning_kokkos import _native as N

    text = open(HEADER).read()
    enum = text[text.index("PLK_GATE_IDENTITY = 0"):text.index("PLK_GATE_COUNT")]
    names = re.findall(r"PLK_GATE_(\w+)", enum)
    assert len(names) == len(N.GATES)
    for i, n in enumerate(N.GATES[:-1]):
        g = C.c_int32(-1)
        assert N.lib.plk_gate_from_name(n.encode(), C.byref(g)) == 0, n
        assert g.value == i
        assert names[i].replace("_", "") == n.upper().replace("_", "")
    g = C.c_int32(0)
    assert N.lib.plk_gate_from_name(b"NotAGate", C.byref(g)) == 2
    assert "NotAGate" in N.last_error()
    assert N.lib.plk_gate_num_wires(N.GATE_ID["Toffoli"]) == 3
    assert N.lib.plk_gate_num_params(N.GATE_ID["Rot"]) == 3
    assert N.lib.plk_gate_num_wires(N.GATE_ID["MultiRZ"]) == -1


def test_module_surface_matches_reference():
    import pennylane_lightning_kokkos.lightning_kokkos_qubit_ops as m

    for bits in ("64", "128"):
        for cls in ("LightningKokkos_C", "ObservableKokkos_C", "NamedObsKokkos_C", "HermitianObsKokkos_C",
                    "TensorProdObsKokkos_C", "HamiltonianKokkos_C", "SparseHamiltonianKokkos_C",
                    "OpsStructKokkos_C", "AdjointJacobianKokkos_C"):
            assert hasattr(m, cls + bits), cls + bits
        sv = getattr(m, "LightningKokkos_C" + bits)
        for meth in ("Identity", "PauliX", "PauliY", "PauliZ", "Hadamard", "S", "T", "CNOT", "SWAP", "CSWAP",
                     "Toffoli", "CY", "CZ", "PhaseShift", "ControlledPhaseShift", "RX", "RY", "RZ", "Rot", "CRX",
                     "CRY", "CRZ", "CRot", "IsingXX", "IsingXY", "IsingYY", "IsingZZ", "MultiRZ",
                     "SingleExcitation", "SingleExcitationMinus", "SingleExcitationPlus", "DoubleExcitation",
                     "DoubleExcitationMinus", "DoubleExcitationPlus", "apply", "applyGenerator",
                     "ExpectationValue", "probs", "GenerateSamples", "DeviceToHost", "HostToDevice",
                     "setBasisState", "setStateVector", "numQubits", "dataLength", "resetKokkos"):
            assert hasattr(sv, meth), meth
        adj = getattr(m, "AdjointJacobianKokkos_C" + bits)
        assert hasattr(adj, "create_ops_list") and hasattr(adj, "adjoint_jacobian")
    for f in ("kokkos_start", "kokkos_end", "kokkos_config_info", "print_configuration", "InitializationSettings",
              "PLException"):
        assert hasattr(m, f)
    s = m.InitializationSettings().set_device_id(0).set_num_threads(4)
    assert s.get_device_id() == 0 and s.get_num_threads() == 4 and s.has_num_threads()


def test_observables_build_without_device():
    import numpy as np
    import pennylane_lightning_kokkos.lightning_kokkos_qubit_ops as m

    z0 = m.NamedObsKokkos_C128("PauliZ", [0])
    x1 = m.NamedObsKokkos_C128("PauliX", [1])
    t = m.TensorProdObsKokkos_C128([z0, x1])
    h = m.HamiltonianKokkos_C128(np.array([0.5, -0.2]), [z0, t])
    assert repr(z0) == "PauliZ[0]"
    assert repr(t) == "PauliZ[0] @ PauliX[1]"
    assert t.get_wires() == [0, 1]
    assert h.get_wires() == [0, 1]
    assert z0 == m.NamedObsKokkos_C128("PauliZ", [0]) and not (z0 == x1)
    with pytest.raises(m.PLException):
        m.TensorProdObsKokkos_C128([z0, m.NamedObsKokkos_C128("PauliX", [0])])  # overlapping wires
    ops = m.AdjointJacobianKokkos_C128().create_ops_list(["RX", "CNOT"], [np.array([0.3]), np.array([])],
                                                          [[0], [0, 1]], [False, False], [np.array([]), np.array([])])
    assert "RX" in repr(ops)


def test_c128_arithmetic_switch():
    # the mode is host state only: set, read back, reject unknown modes, restore
    from pennylane_lightning_kokkos import _native as N

    before = N.c128_arithmetic()
    try:
        N.set_c128_arithmetic("fp64")
        assert N.c128_arithmetic() == "fp64"
        N.set_c128_arithmetic("double-float")
        assert N.c128_arithmetic() == "double-float"
        assert N.lib.plk_set_c128_arithmetic(7) == 1  # PLK_ERR_INVALID_ARG
        assert "arithmetic mode" in N.last_error()
        assert N.c128_arithmetic() == "double-float"
    finally:
        N.set_c128_arithmetic(before)


@pytest.mark.skipif(os.environ.get("CUDA_VISIBLE_DEVICES") is None and os.path.exists("/dev/nvidia0"),
                    reason="a GPU is present")
def test_no_device_fails_loudly():
    import pennylane_lightning_kokkos.lightning_kokkos_qubit_ops as m
    from pennylane_lightning_kokkos import _native as N

    if N.device_count() > 0:
        pytest.skip("a GPU is present")
    with pytest.raises(m.PLException, match="no CUDA device"):
        m.LightningKokkos_C128(3)
    h = C.c_void_p()
    assert N.lib.plk_state_create(3, 1, 0, C.byref(h)) == 6  # PLK_ERR_NO_DEVICE


def test_gate_matrices_match_oracle():
    """plk_gate_matrix (host side of the gate plans, used by the batch engine)
    equals the oracle's gate applied to every basis state."""
    import numpy as np

    import oracle as O
    from pennylane_lightning_kokkos import _native as N

    rng = np.random.default_rng(11)
    for name in N.GATES:
        if name in ("Matrix",):
            continue
        g = N.GATE_ID[name]
        nw = N.lib.plk_gate_num_wires(g)
        for k in ([1, 2, 3] if nw < 0 else [nw]):
            npar = N.lib.plk_gate_num_params(g)
            prm = [float(x) for x in rng.uniform(-np.pi, np.pi, npar)]
            for inv in (False, True):
                M = N.gate_matrix(name, prm, num_wires=k, adjoint=inv)
                ref = np.zeros_like(M)
                for c in range(1 << k):
                    e = O.zero_state(k)
                    e[0] = 0
                    e[c] = 1
                    O.apply(e, name, list(range(k)), inv, prm)
                    ref[:, c] = e
                np.testing.assert_allclose(M, ref, atol=1e-15, err_msg=f"{name} k={k} inv={inv}")


def test_batch_needs_a_device():
    import ctypes as C

    from pennylane_lightning_kokkos import _native as N

    h = C.c_void_p()
    assert N.lib.plk_batch_create(0, 0, C.byref(h)) == 6  # PLK_ERR_NO_DEVICE
    assert "no CUDA device" in N.last_error()
