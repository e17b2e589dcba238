"""Known answers transcribed from the reference's own C++ unit tests.

Every entry cites the test file and line range it was read from (paths
relative to pennylane_lightning_kokkos/src/tests/).  The values are data only;
the tests in ``tests/test_oracle_golden.py`` pin the CPU oracle to them and the
GPU parity tests pin the CUDA path to the oracle.

Complex numbers are written as Python complex literals.  Tolerances are those
of the reference test (Catch2 ``Approx`` default epsilon = 100*FLT_EPSILON
relative, or the stated margin).
"""
import math

# --------------------------------------------------------------------------
# Shared initial states
# --------------------------------------------------------------------------
# Test_StateVectorKokkos_Generator.cpp:25-42 and Test_StateVectorKokkos_Param.cpp:24-41
INI_4Q_A = [
    0.267462841882 + 0.010768564798j, 0.228575129706 + 0.010564590956j,
    0.099492749900 + 0.260849823392j, 0.093690204310 + 0.189847108173j,
    0.033390732374 + 0.203836830144j, 0.226979395737 + 0.081852150975j,
    0.031235505729 + 0.176933497281j, 0.294287602843 + 0.145156781198j,
    0.152742706049 + 0.111628061129j, 0.012553863703 + 0.120027860480j,
    0.237156555364 + 0.154658769755j, 0.117001120872 + 0.228059505033j,
    0.041495873225 + 0.065934827444j, 0.089653239407 + 0.221581340372j,
    0.217892322429 + 0.291261296999j, 0.292993251871 + 0.186570798697j,
]

# Test_StateVectorKokkos_Param.cpp:1128-1145 (DoubleExcitation) and :961-966
INI_4Q_B = [
    0.125681356503 + 0.252712197380j, 0.262591068130 + 0.370189000494j,
    0.129300299863 + 0.371057794075j, 0.392248682814 + 0.195795523118j,
    0.303908059240 + 0.082981563244j, 0.189140284321 + 0.179512645957j,
    0.173146612336 + 0.092249594834j, 0.298857179897 + 0.269627836165j,
] * 2

# Test_StateVectorKokkos_Expval.cpp:368-370 (unnormalised 3-qubit state)
INI_3Q_C = [0.0 + 0.0j, 0.0 + 0.1j, 0.1 + 0.1j, 0.1 + 0.2j,
            0.2 + 0.2j, 0.3 + 0.3j, 0.3 + 0.4j, 0.4 + 0.5j]

# --------------------------------------------------------------------------
# Gate known answers: (initial state or None for |0..0>, nq, ops, expected, rel_tol)
# ops = [(name, wires, inverse, params)]
# --------------------------------------------------------------------------
GATE_CASES = {
    # Test_StateVectorKokkos_Param.cpp:92-148
    "RX_0.1": (None, 1, [("RX", [0], False, [0.1])],
               [0.9987502603949663 + 0.0j, -0.04997916927067834j], 1.2e-5),
    "RX_0.6": (None, 1, [("RX", [0], False, [0.6])],
               [0.9553364891256061 + 0.0j, -0.2955202066613395j], 1.2e-5),
    "RX_adj_0.1": (None, 1, [("RX", [0], True, [0.1])],
                   [0.9987502603949663 + 0.0j, 0.04997916927067834j], 1.2e-5),
    "RX_adj_0.6": (None, 1, [("RX", [0], True, [0.6])],
                   [0.9553364891256061 + 0.0j, 0.2955202066613395j], 1.2e-5),
    # Test_StateVectorKokkos_Param.cpp:18-90 (IsingXY on {0,1}, 0.312)
    "IsingXY": (INI_4Q_A, 4, [("IsingXY", [0, 1], False, [0.312])], [
        0.267462849617 + 0.010768564418j, 0.228575125337 + 0.010564590804j,
        0.099492751062 + 0.260849833488j, 0.093690201640 + 0.189847111702j,
        0.015641822883 + 0.225092900621j, 0.205574608177 + 0.082808663337j,
        0.006827173322 + 0.211631480575j, 0.255280800811 + 0.161572331669j,
        0.119218164572 + 0.115460377284j, -0.000315789761 + 0.153835664378j,
        0.206786872079 + 0.157633689097j, 0.093027614553 + 0.271012980118j,
        0.041495874524 + 0.065934829414j, 0.089653238654 + 0.221581339836j,
        0.217892318964 + 0.291261285543j, 0.292993247509 + 0.186570793390j,
    ], 1.2e-5),
    # Test_StateVectorKokkos_Param.cpp:954-1007 (SingleExcitation on {0,2})
    "SingleExcitation": (INI_4Q_B[:8], 3,
                         [("SingleExcitation", [0, 2], False, [0.267030328057308])], [
        0.125681 + 0.252712j, 0.219798 + 0.355848j, 0.1293 + 0.371058j,
        0.365709 + 0.181773j, 0.336159 + 0.131522j, 0.18914 + 0.179513j,
        0.223821 + 0.117493j, 0.298857 + 0.269628j,
    ], 2e-5),
    # Test_StateVectorKokkos_Param.cpp:1121-1187 (DoubleExcitation on {0,1,2,3})
    "DoubleExcitation": (INI_4Q_B, 4,
                         [("DoubleExcitation", [0, 1, 2, 3], False, [0.267030328057308])], [
        0.125681 + 0.252712j, 0.262591 + 0.370189j, 0.1293 + 0.371058j,
        0.348302 + 0.183007j, 0.303908 + 0.0829816j, 0.18914 + 0.179513j,
        0.173147 + 0.0922496j, 0.298857 + 0.269628j, 0.125681 + 0.252712j,
        0.262591 + 0.370189j, 0.1293 + 0.371058j, 0.392249 + 0.195796j,
        0.353419 + 0.108307j, 0.18914 + 0.179513j, 0.173147 + 0.0922496j,
        0.298857 + 0.269628j,
    ], 2e-5),
}

# Test_StateVectorKokkos_Generator.cpp: wires used for each generator,
# checked as d/dtheta U(theta)|psi> = i * scale * G |psi> by central finite
# differences at ep = 1e-3 with margin 1e-4 on INI_4Q_A.
GENERATOR_WIRES = {
    "PhaseShift": [1], "IsingXX": [0, 1], "IsingXY": [0, 1], "IsingYY": [0, 1],
    "IsingZZ": [0, 1], "ControlledPhaseShift": [0, 1], "CRX": [0, 1],
    "CRY": [0, 1], "CRZ": [0, 1], "MultiRZ": [0], "RX": [1], "RY": [1],
    "RZ": [1], "SingleExcitation": [0, 1], "SingleExcitationMinus": [0, 1],
    "SingleExcitationPlus": [0, 1], "DoubleExcitation": [0, 1, 2, 3],
    "DoubleExcitationMinus": [0, 1, 2, 3], "DoubleExcitationPlus": [0, 1, 2, 3],
}
GENERATOR_FD = (1e-3, 1e-4)  # (ep, margin)

# --------------------------------------------------------------------------
# Probabilities: Test_StateVectorKokkos_Measure.cpp:19-62 on the state of
# TestHelpers.hpp:153-177 (RX, RY on each wire, phases 0.7, 0.5, 0.3), margin 1e-6
# --------------------------------------------------------------------------
PROBS_INIT_OPS = [("RX", [0], False, [0.7]), ("RY", [0], False, [0.7]),
                  ("RX", [1], False, [0.5]), ("RY", [1], False, [0.5]),
                  ("RX", [2], False, [0.3]), ("RY", [2], False, [0.3])]
PROBS_CASES = [
    ([0, 1, 2], [0.67078706, 0.03062806, 0.0870997, 0.00397696, 0.17564072, 0.00801973, 0.02280642, 0.00104134]),
    ([0, 2, 1], [0.67078706, 0.0870997, 0.03062806, 0.00397696, 0.17564072, 0.02280642, 0.00801973, 0.00104134]),
    ([1, 0, 2], [0.67078706, 0.03062806, 0.17564072, 0.00801973, 0.0870997, 0.00397696, 0.02280642, 0.00104134]),
    ([1, 2, 0], [0.67078706, 0.0870997, 0.17564072, 0.02280642, 0.03062806, 0.00397696, 0.00801973, 0.00104134]),
    ([2, 0, 1], [0.67078706, 0.17564072, 0.03062806, 0.00801973, 0.0870997, 0.02280642, 0.00397696, 0.00104134]),
    ([2, 1, 0], [0.67078706, 0.17564072, 0.0870997, 0.02280642, 0.03062806, 0.00801973, 0.00397696, 0.00104134]),
    ([0, 1], [0.70141512, 0.09107666, 0.18366045, 0.02384776]),
    ([0, 2], [0.75788676, 0.03460502, 0.19844714, 0.00906107]),
    ([1, 2], [0.84642778, 0.0386478, 0.10990612, 0.0050183]),
    ([2, 1], [0.84642778, 0.10990612, 0.0386478, 0.0050183]),
    ([0], [0.79249179, 0.20750821]),
    ([1], [0.88507558, 0.11492442]),
    ([2], [0.9563339, 0.0436661]),
]
PROBS_MARGIN = 1e-6
# Test_StateVectorKokkos_Param.cpp:1325-1394: 100000 samples, histogram within 0.05
SAMPLE_SHOTS, SAMPLE_MARGIN = 100000, 0.05

# --------------------------------------------------------------------------
# Expectation values and variances
# --------------------------------------------------------------------------
# Test_StateVectorKokkos_Expval.cpp:366-421: 8x8 (non-Hermitian) matrix, Re part 1.263
# matrix literal at :373-386, 64 entries, row-major
HERMITIAN_3Q_MATRIX = (
    [0.5, 0.2 + 0.5j, 0.2 - 0.5j, 0.3, 0.2 - 0.5j, 0.3, 0.2 - 0.5j, 0.3,
     0.2 - 0.5j, 0.3, 0.2 - 0.5j, 0.3, 0.2 - 0.5j, 0.3, 0.2 - 0.5j, 0.3,
     0.5, 0.2 + 0.5j, 0.2 - 0.5j, 0.3, 0.2 - 0.5j, 0.3, 0.2 - 0.5j, 0.3,
     0.2 - 0.5j, 0.3, 0.2 - 0.5j, 0.3, 0.2 - 0.5j, 0.3, 0.2 - 0.5j, 0.3,
     0.5, 0.2 + 0.5j, 0.2 - 0.5j, 0.3, 0.2 - 0.5j, 0.3, 0.2 - 0.5j, 0.3,
     0.2 - 0.5j, 0.3, 0.2 - 0.5j, 0.3, 0.2 - 0.5j, 0.3, 0.2 - 0.5j, 0.3,
     0.5, 0.2 + 0.5j, 0.2 - 0.5j, 0.3, 0.2 - 0.5j, 0.3, 0.2 - 0.5j, 0.3,
     0.2 - 0.5j, 0.3, 0.2 - 0.5j, 0.3, 0.2 - 0.5j, 0.3, 0.2 - 0.5j, 0.3])
EXPVAL_HERMITIAN_3Q = 1.263
# :423-447 CSR sparse Hamiltonian, expected 3.1415
SPARSE_INDPTR = [0, 2, 4, 6, 8, 10, 12, 14, 16]
SPARSE_INDICES = [0, 3, 1, 2, 1, 2, 0, 3, 4, 7, 5, 6, 5, 6, 4, 7]
_p = 3.1415
SPARSE_VALUES = [_p, -_p * 1j, _p, _p * 1j, -_p * 1j, _p, _p * 1j, _p,
                 _p, -_p * 1j, _p, _p * 1j, -_p * 1j, _p, _p * 1j, _p]
EXPVAL_SPARSE = 3.1415
# :449-469 Hamiltonian 0.3 X0 + 0.5 Z1 on INI_3Q_C -> -0.086
EXPVAL_HAMILTONIAN = -0.086
# :471-491 Tensor X0 @ Z1 on INI_3Q_C -> -0.36
EXPVAL_TENSOR = -0.36

# Test_LinearAlgebra.cpp:10-52 SpMV with unit values
SPMV_X = INI_3Q_C
SPMV_VALUES = [1, -1j, 1, 1j, -1j, 1, 1j, 1, 1, -1j, 1, 1j, -1j, 1, 1j, 1]
SPMV_RESULT = [0.2 - 0.1j, -0.1 + 0.2j, 0.2 + 0.1j, 0.1 + 0.2j,
               0.7 - 0.2j, -0.1 + 0.6j, 0.6 + 0.1j, 0.2 + 0.7j]
# Test_LinearAlgebra.cpp:53-90 axpy: y += (2+0.5i) x
AXPY_ALPHA = 2.0 + 0.5j
AXPY_X = [0, 0.1 - 0.1j, 0.1 + 0.1j, 0.2 + 0.1j, 0.2 + 0.2j, 0.3 + 0.3j, 0.4 + 0.3j, 0.5 + 0.4j]
AXPY_Y = [-0.1 + 0.2j, 0.2 - 0.1j, 0.1 + 0.2j, 0.2 + 0.1j, -0.2 + 0.7j, 0.6 - 0.1j, 0.1 + 0.6j, 0.7 + 0.2j]
AXPY_RESULT = [-0.1 + 0.2j, 0.45 - 0.25j, 0.25 + 0.45j, 0.55 + 0.4j,
               0.1 + 1.2j, 1.05 + 0.65j, 0.75 + 1.4j, 1.5 + 1.25j]

# Test_StateVectorKokkos_Var.cpp:19-160
VAR_2Q_OPS = [("RX", [0], False, [0.7]), ("RY", [0], False, [0.7]),
              ("RX", [1], False, [0.5]), ("RY", [1], False, [0.5])]
VAR_NAMED = [(("named", "PauliX", [0]), 0.7572222074),
             (("named", "PauliY", [0]), 0.5849835715),
             (("named", "PauliZ", [1]), 0.4068672016)]
VAR_3Q_OPS = VAR_2Q_OPS + [("RX", [2], False, [0.3]), ("RY", [2], False, [0.3])]
_th = math.pi / 2
_c, _js = math.cos(_th / 2), math.sin(-_th / 2)
VAR_HERMITIAN_MATRIX = [0j] * 16
VAR_HERMITIAN_MATRIX[0] = _c
VAR_HERMITIAN_MATRIX[1] = 1j * _js
VAR_HERMITIAN_MATRIX[4] = 1j * _js
VAR_HERMITIAN_MATRIX[5] = _c
VAR_HERMITIAN_MATRIX[10] = 1
VAR_HERMITIAN_MATRIX[15] = 1
VAR_HERMITIAN = 0.4103533486  # wires {0, 2}
VAR_TENSOR_OPS = [("RX", [0], False, [0.5]), ("RY", [0], False, [0.5]),
                  ("RX", [1], False, [0.2]), ("RY", [1], False, [0.2])]
VAR_TENSOR = 0.836679  # X0 @ Z1 on 3 qubits
VAR_HAMILTONIAN = 0.224604  # 0.3 X0 + 0.5 Z1 on INI_3Q_C

# --------------------------------------------------------------------------
# Adjoint Jacobians: Test_AdjointDiffKokkos.cpp
# (initial state or None, nq, ops, observables, trainable, expected, margin)
# --------------------------------------------------------------------------
_P = [-math.pi / 7, math.pi / 5, 2 * math.pi / 3]
ADJOINT_CASES = {}
for _i, _p in enumerate(_P):
    # :30-60 Op=RX, Obs=Z: -sin(p)
    ADJOINT_CASES[f"RX_Z_{_i}"] = (None, 1, [("RX", [0], False, [_p])], [("named", "PauliZ", [0])],
                                   [0], [[-math.sin(_p)]], 1e-5)
    # :62-85 Op=RY, Obs=X: cos(p)
    ADJOINT_CASES[f"RY_X_{_i}"] = (None, 1, [("RY", [0], False, [_p])], [("named", "PauliX", [0])],
                                   [0], [[math.cos(_p)]], 1e-5)
_RXRXRX = [("RX", [0], False, [_P[0]]), ("RX", [1], False, [_P[1]]), ("RX", [2], False, [_P[2]])]
_Z = [("named", "PauliZ", [w]) for w in range(3)]
# :87-115 Op=RX on 2 qubits, Obs=[Z0,Z1]
ADJOINT_CASES["RX_ZZ"] = (None, 2, [("RX", [0], False, [_P[0]])], _Z[:2], [0],
                          [[-math.sin(_P[0])], [0.0]], 1e-7)
# :117-146 [RX,RX,RX], Obs=[Z,Z,Z] (diagonal checked)
ADJOINT_CASES["RXRXRX_ZZZ"] = (None, 3, _RXRXRX, _Z, [0, 1, 2],
                               [[-math.sin(_P[0]), None, None], [None, -math.sin(_P[1]), None],
                                [None, None, -math.sin(_P[2])]], 1e-7)
# :148-176 TParams=[0,2]
ADJOINT_CASES["RXRXRX_ZZZ_tp02"] = (None, 3, _RXRXRX, _Z, [0, 2],
                                    [[-math.sin(_P[0]), None], [None, 0.0], [None, -math.sin(_P[2])]], 1e-7)
# :178-212 Obs = Z@Z@Z
ADJOINT_CASES["RXRXRX_ZZZtensor"] = (None, 3, _RXRXRX, [("tensor", _Z)], [0, 1, 2],
                                     [[-0.1755096592645253, 0.26478810666384334, -0.6312451595102775]], 1e-7)
# :214-260 Mixed ops, Obs = X@X@X
_MIXED = [("RZ", [0], False, [_P[0]]), ("RY", [0], False, [_P[1]]), ("RZ", [0], False, [_P[2]]),
          ("CNOT", [0, 1], False, []), ("CNOT", [1, 2], False, []),
          ("RZ", [1], False, [_P[0]]), ("RY", [1], False, [_P[1]]), ("RZ", [1], False, [_P[2]])]
ADJOINT_CASES["Mixed_XXX"] = (None, 3, _MIXED, [("tensor", [("named", "PauliX", [w]) for w in range(3)])],
                              [0, 1, 2, 3, 4, 5],
                              [[0.0, -0.674214427, 0.275139672, 0.275139672, -0.0129093062, 0.323846156]],
                              1e-7)
# :262-317 decomposed Rot on [1/sqrt2, -1/sqrt2], Obs = Z0
_thetas = [-2 * math.pi + i * (4 * math.pi / 6) for i in range(7)]
_rot_expected = [[0, -9.90819496e-01, 0], [-8.18996553e-01, 1.62526544e-01, 0], [-0.203949, 0.48593716, 0],
                 [0, 1, 0], [-2.03948985e-01, 4.85937177e-01, 0], [-8.18996598e-01, 1.62526487e-01, 0],
                 [0, -9.90819511e-01, 0]]
for _i, (_t, _e) in enumerate(zip(_thetas, _rot_expected)):
    _lp = [_t, _t ** 3, math.sqrt(2) * _t]
    ADJOINT_CASES[f"Rot_decomposed_{_i}"] = (
        [1 / math.sqrt(2), -1 / math.sqrt(2)], 1,
        [("RZ", [0], False, [_lp[0]]), ("RY", [0], False, [_lp[1]]), ("RZ", [0], False, [_lp[2]])],
        [("named", "PauliZ", [0])], [0, 1, 2], [_e], 1e-6)
# :319-390 Mixed ops, Obs = X0@Z1, TParams=[1,2,3] on |00>
_lp = [0.543, 0.54, 0.1, 0.5, 1.3, -2.3, 0.5, -0.5, 0.5]
_MIXED2 = [("Hadamard", [0], False, []), ("RX", [0], False, [_lp[0]]), ("CNOT", [0, 1], False, []),
           ("RZ", [0], False, [_lp[1]]), ("RY", [0], False, [_lp[2]]), ("RZ", [0], False, [_lp[3]]),
           ("RZ", [0], False, [_lp[4]]), ("RY", [0], False, [_lp[5]]), ("RZ", [0], False, [_lp[6]]),
           ("RZ", [0], False, [_lp[7]]), ("RY", [1], False, [_lp[8]]), ("CNOT", [0, 1], False, [])]
ADJOINT_CASES["Mixed_XZ_tp123"] = (None, 2, _MIXED2,
                                   [("tensor", [("named", "PauliX", [0]), ("named", "PauliZ", [1])])],
                                   [1, 2, 3], [[-0.71429188, 0.04998561, -0.71904837]], 2e-5)
# :392-418 Obs = Ham(0.3 Z0 + 0.7 Z1)
ADJOINT_CASES["RX_Ham2"] = (None, 2, [("RX", [0], False, [_P[0]])],
                            [("hamiltonian", [0.3, 0.7], _Z[:2])], [0], [[-0.3 * math.sin(_P[0])]], 1e-7)
# :420-455 Obs = Ham(0.47 Z0 + 0.32 Z1 + 0.96 Z2), TParams=[0,2]
ADJOINT_CASES["RXRXRX_Ham3_tp02"] = (None, 3, _RXRXRX, [("hamiltonian", [0.47, 0.32, 0.96], _Z)], [0, 2],
                                     [[-0.47 * math.sin(_P[0]), -0.96 * math.sin(_P[2])]], 1e-7)
# :457-491 Hermitian diag(1,-1,-1,1) on {0,1} == Z0@Z1
ADJOINT_HERMITIAN_EQ_TENSOR = (
    3, _RXRXRX, ("tensor", _Z[:2]),
    ("hermitian", [1, 0, 0, 0, 0, -1, 0, 0, 0, 0, -1, 0, 0, 0, 0, 1], [0, 1]), [0, 2], 1e-7)
