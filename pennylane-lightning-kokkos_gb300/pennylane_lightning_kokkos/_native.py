"""ctypes view of the C ABI in ``include/plk_gb300.h`` (``libplk_gb300.so``).

The pybind11 module ``lightning_kokkos_qubit_ops`` is the reference-facing
interface; this module exposes the same kernels through plain pointers for
code that manages device memory itself (the torch autograd layer, the batched
circuit runner) and for tests that check the ABI.  There is no fallback: if
the library is missing, importing this module raises ImportError.
"""
from __future__ import annotations

import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libplk_gb300.so")

if not os.path.exists(LIB_PATH):
    raise ImportError(
        f"{LIB_PATH} is missing: build the GB300 core first "
        "(python pennylane-lightning-kokkos_gb300/build.py)")

lib = C.CDLL(LIB_PATH)

PLK_OK = 0
PLK_C64, PLK_C128 = 0, 1
PLK_ARITH_DOUBLE_FLOAT, PLK_ARITH_FP64 = 0, 1
STATUS_NAMES = {0: "OK", 1: "INVALID_ARG", 2: "UNKNOWN_GATE", 3: "CUDA", 4: "OUT_OF_MEMORY", 5: "UNSUPPORTED",
                6: "NO_DEVICE"}

GATES = ["Identity", "PauliX", "PauliY", "PauliZ", "Hadamard", "S", "T", "PhaseShift", "RX", "RY", "RZ", "Rot",
         "CNOT", "CY", "CZ", "SWAP", "ControlledPhaseShift", "CRX", "CRY", "CRZ", "CRot", "IsingXX", "IsingXY",
         "IsingYY", "IsingZZ", "SingleExcitation", "SingleExcitationMinus", "SingleExcitationPlus",
         "DoubleExcitation", "DoubleExcitationMinus", "DoubleExcitationPlus", "CSWAP", "Toffoli", "MultiRZ",
         "Matrix"]
GATE_ID = {n: i for i, n in enumerate(GATES)}
GATE_MATRIX = GATE_ID["Matrix"]


class NativeError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"[{STATUS_NAMES.get(status, status)}] {msg}")
        self.status = status


class PlkOp(C.Structure):
    _fields_ = [("gate", C.c_int32), ("num_wires", C.c_int32), ("adjoint", C.c_int32), ("num_params", C.c_int32),
                ("wires", C.POINTER(C.c_int64)), ("params", C.POINTER(C.c_double)),
                ("matrix", C.POINTER(C.c_double))]


class PlkDeviceInfo(C.Structure):
    _fields_ = [("device", C.c_int), ("sm_count", C.c_int), ("cc_major", C.c_int), ("cc_minor", C.c_int),
                ("total_mem", C.c_uint64), ("free_mem", C.c_uint64), ("clock_khz", C.c_int),
                ("mem_clock_khz", C.c_int), ("mem_bus_width", C.c_int), ("name", C.c_char * 128)]


_vp, _i64p, _dp, _i32p = C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_double), C.POINTER(C.c_int32)
_SIGS = {
    "plk_last_error": ([], C.c_char_p),
    "plk_version": ([], C.c_int),
    "plk_device_count": ([C.POINTER(C.c_int)], C.c_int),
    "plk_get_device_info": ([C.c_int, C.POINTER(PlkDeviceInfo)], C.c_int),
    "plk_gate_from_name": ([C.c_char_p, _i32p], C.c_int),
    "plk_gate_num_wires": ([C.c_int32], C.c_int),
    "plk_gate_num_params": ([C.c_int32], C.c_int),
    "plk_state_create": ([C.c_int, C.c_int, C.c_int, C.POINTER(_vp)], C.c_int),
    "plk_state_wrap": ([_vp, C.c_int, C.c_int, C.c_int, _vp, C.POINTER(_vp)], C.c_int),
    "plk_state_destroy": ([_vp], C.c_int),
    "plk_state_get": ([_vp, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(_vp)], C.c_int),
    "plk_state_set_stream": ([_vp, _vp], C.c_int),
    "plk_state_get_stream": ([_vp, C.POINTER(_vp)], C.c_int),
    "plk_state_synchronize": ([_vp], C.c_int),
    "plk_state_reset": ([_vp], C.c_int),
    "plk_state_zero": ([_vp], C.c_int),
    "plk_state_set_basis": ([_vp, C.c_uint64], C.c_int),
    "plk_state_set_values": ([_vp, C.POINTER(C.c_uint64), _vp, C.c_uint64], C.c_int),
    "plk_state_h2d": ([_vp, _vp, C.c_uint64], C.c_int),
    "plk_state_d2h": ([_vp, _vp, C.c_uint64], C.c_int),
    "plk_state_h2d_async": ([_vp, _vp, C.c_uint64], C.c_int),
    "plk_state_d2h_async": ([_vp, _vp, C.c_uint64], C.c_int),
    "plk_state_copy": ([_vp, _vp], C.c_int),
    "plk_state_axpy": ([_vp, C.c_double, C.c_double, _vp], C.c_int),
    "plk_apply_gate": ([_vp, C.c_int32, _i64p, C.c_int32, C.c_int32, _dp, C.c_int32], C.c_int),
    "plk_apply_matrix": ([_vp, _dp, _i64p, C.c_int32, C.c_int32], C.c_int),
    "plk_apply_ops": ([_vp, C.POINTER(PlkOp), C.c_int32], C.c_int),
    "plk_apply_generator": ([_vp, C.c_int32, _i64p, C.c_int32, C.c_int32, _dp], C.c_int),
    "plk_expval_named": ([_vp, C.c_int32, _i64p, C.c_int32, _dp], C.c_int),
    "plk_expval_named_batch": ([_vp, C.c_int32, _i32p, _i64p, _dp], C.c_int),
    "plk_expval_matrix": ([_vp, _dp, _i64p, C.c_int32, _dp], C.c_int),
    "plk_expval_sparse": ([_vp, _dp, _i64p, _i64p, C.c_int64, C.c_int64, _dp], C.c_int),
    "plk_expval_pauli_sum": ([_vp, C.c_int32, _dp, _i64p, _i64p, C.c_char_p, _dp], C.c_int),
    "plk_apply_pauli_sum": ([_vp, _vp, C.c_int32, _dp, _i64p, _i64p, C.c_char_p], C.c_int),
    "plk_inner_product": ([_vp, _vp, _dp, _dp], C.c_int),
    "plk_spmv": ([_vp, _vp, _dp, _i64p, _i64p, C.c_int64, C.c_int64], C.c_int),
    "plk_probs": ([_vp, _i64p, C.c_int32, _dp], C.c_int),
    "plk_cdf": ([_vp, _dp], C.c_int),
    "plk_sample_from_uniforms": ([_vp, _dp, C.c_uint64, _i64p], C.c_int),
    "plk_search_cdf": ([_dp, C.c_uint64, C.c_int32, _dp, C.c_uint64, _i64p, C.c_int], C.c_int),
    "plk_generate_samples": ([_vp, C.c_uint64, C.c_uint64, _i64p], C.c_int),
    "plk_adjoint_jacobian": ([_vp, C.POINTER(_vp), C.c_int32, C.POINTER(PlkOp), C.c_int32, _i64p, C.c_int32, _dp],
                             C.c_int),
    "plk_adjoint_jacobian_inplace": ([_vp, C.POINTER(_vp), C.c_int32, C.POINTER(PlkOp), C.c_int32, _i64p, C.c_int32,
                                      _dp], C.c_int),
    "plk_expval_pauliz_noalloc": ([_vp, C.c_int32, C.c_int32, C.c_int32, _i64p, _dp, _vp], C.c_int),
    "plk_set_window_path": ([C.c_int32], C.c_int),
    "plk_get_window_path": ([_i32p], C.c_int),
    "plk_set_c128_arithmetic": ([C.c_int32], C.c_int),
    "plk_set_dense_tensor_cores": ([C.c_int32], C.c_int),
    "plk_get_dense_tensor_cores": ([_i32p], C.c_int),
    "plk_get_c128_arithmetic": ([_i32p], C.c_int),
    "plk_gate_matrix": ([C.c_int32, _dp, C.c_int32, C.c_int32, C.c_int32, _dp], C.c_int),
    "plk_batch_create": ([C.c_int32, C.c_int32, C.POINTER(_vp)], C.c_int),
    "plk_batch_destroy": ([_vp], C.c_int),
    "plk_batch_add": ([_vp, C.c_int32, C.POINTER(PlkOp), C.c_int32, _i64p, C.c_int32, C.c_int32, _dp, _i64p, _i64p,
                       C.c_char_p, _i64p], C.c_int),
    "plk_batch_info": ([_vp, _i64p, _i64p, _i64p], C.c_int),
    "plk_batch_circuit_info": ([_vp, C.c_int64, _i64p, _i32p, _i64p, _i32p], C.c_int),
    "plk_batch_set_params": ([_vp, _dp, C.c_int64], C.c_int),
    "plk_batch_run": ([_vp, _dp, _dp], C.c_int),
    "plk_batch_run_device": ([_vp, _dp, _dp, _dp, _vp], C.c_int),
    "plk_batch_last_time": ([_vp, _dp, _i64p], C.c_int),
    "plk_batch_set_config": ([_vp, C.c_int32, C.c_int32, C.c_int32, C.c_int32], C.c_int),
    "plk_batch_get_config": ([_vp, _i32p, _i32p, _i32p, _i32p], C.c_int),
    "plk_batch_set_graph": ([_vp, C.c_int32], C.c_int),
    "plk_batch_set_occupancy": ([_vp, C.c_int32], C.c_int),
    "plk_batch_get_occupancy": ([_vp, _i32p], C.c_int),
    "plk_batch_tune": ([_vp, C.c_int32, C.c_char_p, C.c_int32], C.c_int),
}
for _name, (_args, _res) in _SIGS.items():
    _f = getattr(lib, _name)
    _f.argtypes = _args
    _f.restype = _res


def last_error() -> str:
    return lib.plk_last_error().decode(errors="replace")


def check(status: int) -> None:
    if status != PLK_OK:
        raise NativeError(status, last_error())


def device_count() -> int:
    n = C.c_int(0)
    check(lib.plk_device_count(C.byref(n)))
    return n.value


def gate_matrix(name: str, params=(), num_wires: int | None = None, adjoint: bool = False):
    """Dense matrix (numpy complex128, wires[0] = most significant bit) of a named gate."""
    import numpy as np

    g = GATE_ID[name]
    nw = num_wires if num_wires is not None else lib.plk_gate_num_wires(g)
    prm = np.ascontiguousarray(np.asarray(list(params) + [0.0] * 3, dtype=np.float64))
    out = np.zeros(2 * (1 << (2 * nw)), dtype=np.float64)
    check(lib.plk_gate_matrix(g, prm.ctypes.data_as(_dp), len(prm), int(adjoint), nw, out.ctypes.data_as(_dp)))
    return out.view(np.complex128).reshape(1 << nw, 1 << nw)


def c128_arithmetic() -> str:
    """'double-float' (FP32 pipe, the default) or 'fp64' (native IEEE double)."""
    m = C.c_int32()
    check(lib.plk_get_c128_arithmetic(C.byref(m)))
    return "fp64" if m.value == PLK_ARITH_FP64 else "double-float"


def set_c128_arithmetic(mode: str) -> None:
    """Select how complex128 kernels compute: 'double-float' or 'fp64'."""
    if mode not in ("double-float", "fp64"):
        raise ValueError("mode must be 'double-float' or 'fp64'")
    check(lib.plk_set_c128_arithmetic(PLK_ARITH_FP64 if mode == "fp64" else PLK_ARITH_DOUBLE_FLOAT))


def device_info(device: int = 0) -> dict:
    info = PlkDeviceInfo()
    check(lib.plk_get_device_info(device, C.byref(info)))
    return {f: (getattr(info, f).decode() if f == "name" else getattr(info, f)) for f, _ in PlkDeviceInfo._fields_}
